// Row preparation kernels: zero padding, the internal GF checksum (compute on
// inputs, verify on outputs), PAR2 coefficient expansion into the
// combination-table index layout, and the seeded synthetic data generator.
//
// Checksum (same value as the reference's generic 8-byte checksum,
// gf16/gf16_checksum_generic.h:25-130 + gf16/gf16_cksum_base.h:32-60):
//   four 16-bit lanes; over the row's 8-byte blocks b = 0..nb-1 (data
//   zero-padded to Sp bytes), ck = sum_b 2^(nb-1-b) * block_b per lane
//   (Horner: ck = 2*ck ^ block).  The product is linear, so the recovery row's
//   carried checksum equals the checksum of its data iff nothing was corrupted.
#include "common.cuh"
#include "kernels.h"

namespace p2c {

// ---- per-row partial checksum + zero tail ----------------------------------
// grid: (rows, splits); each CTA owns a contiguous, 32-byte-aligned part of the
// row's data and folds its partial checksum, pre-multiplied by 2^(blocks after
// it), into ckAcc[row] with a 64-bit atomic XOR.  Bytes at or beyond
// lens[row] are treated as zero and, when zeroTail is set, written as zero
// (each byte is owned by exactly one thread, so there is no race).
__global__ void __launch_bounds__(256) k_rows_cksum_partial(
	uint16_t* rows, size_t pitchWords, const uint32_t* lens, uint32_t fixedLen,
	size_t sliceBytes, unsigned long long* ckAcc, int zeroTail, GfTables gt)
{
	const unsigned row = blockIdx.x;
	const size_t Sp = round_up_dev(sliceBytes, 8);
	const size_t nb = Sp / 8;                // checksum blocks in the row
	const size_t nUnits = (Sp + 31) / 32;    // 32-byte units (4 blocks)
	const size_t perCta = (nUnits + gridDim.y - 1) / gridDim.y;
	const size_t u0 = (size_t)blockIdx.y * perCta;
	const size_t u1 = min(nUnits, u0 + perCta);
	const size_t perThr = (u1 > u0) ? (u1 - u0 + blockDim.x - 1) / blockDim.x : 0;
	const size_t t0 = u0 + (size_t)threadIdx.x * perThr;
	const size_t t1 = min(u1, t0 + perThr);
	const size_t len = lens ? lens[row] : fixedLen;
	uint8_t* base = reinterpret_cast<uint8_t*>(rows + (size_t)row * pitchWords);

	uint32_t hLo = 0, hHi = 0; // lanes 0-1 and 2-3 of the running Horner value
	size_t lastBlock = 0;
	for(size_t u = t0; u < t1; u++) {
		uint4* p = reinterpret_cast<uint4*>(base + u * 32);
		uint4 a = p[0], b = p[1];
		const size_t byte0 = u * 32;
		if(byte0 + 32 > len) {
			// mask bytes >= len to zero
			uint32_t w[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
			for(int q = 0; q < 8; q++) {
				size_t s = byte0 + 4 * q;
				uint32_t keep;
				if(s >= len) keep = 0;
				else if(s + 4 <= len) keep = 0xFFFFFFFFu;
				else keep = 0xFFFFFFFFu >> (8 * (4 - (len - s)));
				w[q] &= keep;
			}
			a = make_uint4(w[0], w[1], w[2], w[3]);
			b = make_uint4(w[4], w[5], w[6], w[7]);
			if(zeroTail) { p[0] = a; p[1] = b; }
		}
		uint32_t blk[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
		for(int k = 0; k < 4; k++) {
			if(u * 4 + k < nb) {
				hLo = mul2x2(hLo) ^ blk[2 * k];
				hHi = mul2x2(hHi) ^ blk[2 * k + 1];
				lastBlock = u * 4 + k + 1;
			}
		}
	}
	uint64_t h = ((uint64_t)hHi << 32) | hLo;
	if(t1 > t0 && h) h = cksum_mul_exp(gt, h, (uint32_t)((nb - lastBlock) % 65535));
	// CTA-wide XOR reduction
#pragma unroll
	for(int off = 16; off; off >>= 1) h ^= __shfl_xor_sync(0xFFFFFFFFu, h, off);
	__shared__ uint64_t red[32];
	if((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = h;
	__syncthreads();
	if(threadIdx.x < 32) {
		h = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0;
#pragma unroll
		for(int off = 16; off; off >>= 1) h ^= __shfl_xor_sync(0xFFFFFFFFu, h, off);
		if(threadIdx.x == 0 && h) atomicXor(ckAcc + row, (unsigned long long)h);
	}
}

// writes the accumulated checksum into the row's checksum block and zeroes the
// pitch padding after it; or (verify) compares it with the carried block
__global__ void k_rows_cksum_finish(uint16_t* rows, size_t pitchWords, unsigned nRows, size_t sliceBytes,
                                    const unsigned long long* ckAcc, int verify, uint8_t* flags)
{
	const unsigned row = blockIdx.x;
	if(row >= nRows) return;
	const size_t Sp = round_up_dev(sliceBytes, 8);
	uint16_t* r = rows + (size_t)row * pitchWords;
	const size_t ckWord = Sp / 2;
	if(verify) {
		if(threadIdx.x == 0) {
			uint64_t carried = 0;
			for(int l = 0; l < 4; l++) carried |= (uint64_t)r[ckWord + l] << (16 * l);
			flags[row] = carried == ckAcc[row] ? 1 : 0;
		}
		return;
	}
	for(size_t w = ckWord + threadIdx.x; w < pitchWords; w += blockDim.x) {
		uint16_t v = 0;
		if(w < ckWord + 4) v = (uint16_t)(ckAcc[row] >> (16 * (w - ckWord)));
		r[w] = v;
	}
}

int rows_cksum(uint16_t* rows, size_t pitchWords, unsigned nRows, const uint32_t* dLens, size_t sliceBytes,
               unsigned long long* dCkAcc, int verify, uint8_t* dFlags, const GfTables& gt, cudaStream_t st)
{
	if(!nRows) return 0;
	P2C_CUDA_TRY(cudaMemsetAsync(dCkAcc, 0, sizeof(unsigned long long) * nRows, st));
	const size_t Sp = round_up(sliceBytes, 8);
	const size_t units = (Sp + 31) / 32;
	// ~64 KiB of row data per CTA, at most 64 CTAs per row
	unsigned splits = (unsigned)std::min<size_t>(64, std::max<size_t>(1, units / 2048));
	dim3 grid(nRows, splits);
	k_rows_cksum_partial<<<grid, 256, 0, st>>>(rows, pitchWords, dLens, (uint32_t)sliceBytes, sliceBytes,
	                                           dCkAcc, verify ? 0 : 1, gt);
	P2C_CUDA_TRY(cudaGetLastError());
	k_rows_cksum_finish<<<nRows, 64, 0, st>>>(rows, pitchWords, nRows, sliceBytes, dCkAcc, verify, dFlags);
	P2C_CUDA_TRY(cudaGetLastError());
	return 0;
}

// ---- coefficient expansion ---------------------------------------------------
// For recovery row r and input group g (inputs 8g..8g+7) writes 16 index bytes:
// byte k = sum_t bit_k(c(r, 8g+t)) << t.  Coefficients come either from PAR2
// logs (c = 2^(log_i * e_r mod 65535), gf16/gfmat_coeff.c:60-77) or from an
// explicit [input][R] matrix (addInput with coefficients).
__global__ void k_make_idx(const uint16_t* inLogs, const uint16_t* custom, const uint16_t* outExp,
                           unsigned R, unsigned nIn, unsigned G, uint4* idx, uint16_t* coeffOut, GfTables gt)
{
	const size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
	if(id >= (size_t)R * G) return;
	const unsigned r = (unsigned)(id / G), g = (unsigned)(id % G);
	uint32_t q[4] = {0, 0, 0, 0};
#pragma unroll
	for(int t = 0; t < 8; t++) {
		unsigned i = g * 8 + t;
		uint32_t c = 0;
		if(i < nIn) {
			if(custom) c = custom[(size_t)i * R + r];
			else c = gt.exp[((uint32_t)inLogs[i] * outExp[r]) % 65535u];
			if(coeffOut) coeffOut[(size_t)r * nIn + i] = (uint16_t)c;
		}
#pragma unroll
		for(int k = 0; k < 16; k++) q[k >> 2] |= ((c >> k) & 1u) << (8 * (k & 3) + t);
	}
	idx[(size_t)r * G + g] = make_uint4(q[0], q[1], q[2], q[3]);
}

int make_idx(const uint16_t* dInLogs, const uint16_t* dCustom, const uint16_t* dOutExp, unsigned R, unsigned nIn,
             uint4* dIdx, uint16_t* dCoeffOut, const GfTables& gt, cudaStream_t st)
{
	unsigned G = (nIn + 7) / 8;
	size_t n = (size_t)R * G;
	if(!n) return 0;
	k_make_idx<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(dInLogs, dCustom, dOutExp, R, nIn, G, dIdx, dCoeffOut, gt);
	P2C_CUDA_TRY(cudaGetLastError());
	return 0;
}

// PAR2 coefficients straight from input numbers and exponents -> index layout
// (no host coefficient matrix: c = 2^(log(num_i) * e_r mod 65535))
__global__ void k_par2_idx(const uint16_t* nums, const uint16_t* outExp, unsigned R, unsigned nIn, unsigned G, uint4* idx,
                           GfTables gt)
{
	const size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
	if(id >= (size_t)R * G) return;
	const unsigned r = (unsigned)(id / G), g = (unsigned)(id % G);
	const uint32_t e = outExp[r];
	uint32_t q[4] = {0, 0, 0, 0};
#pragma unroll
	for(int t = 0; t < 8; t++) {
		unsigned i = g * 8 + t;
		uint32_t c = i < nIn ? gt.exp[((uint32_t)gt.inLog[nums[i] & 32767] * e) % 65535u] : 0;
#pragma unroll
		for(int k = 0; k < 16; k++) q[k >> 2] |= ((c >> k) & 1u) << (8 * (k & 3) + t);
	}
	idx[(size_t)r * G + g] = make_uint4(q[0], q[1], q[2], q[3]);
}

int par2_idx(const uint16_t* dNums, const uint16_t* dExp, unsigned R, unsigned nIn, uint4* dIdx, const GfTables& gt,
             cudaStream_t st)
{
	unsigned G = (nIn + 7) / 8;
	size_t n = (size_t)R * G;
	if(!n) return 0;
	k_par2_idx<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(dNums, dExp, R, nIn, G, dIdx, gt);
	P2C_CUDA_TRY(cudaGetLastError());
	return 0;
}

// the PAR2 coefficient matrix [R][nIn] itself, from input numbers and
// exponents (for the methods that read coefficients rather than index bytes)
__global__ void k_par2_coeffs(const uint16_t* nums, const uint16_t* outExp, unsigned R, unsigned nIn, uint16_t* coeff,
                              GfTables gt)
{
	const size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
	if(id >= (size_t)R * nIn) return;
	const unsigned r = (unsigned)(id / nIn), i = (unsigned)(id % nIn);
	coeff[id] = gt.exp[((uint32_t)gt.inLog[nums[i] & 32767] * outExp[r]) % 65535u];
}

int par2_coeffs(const uint16_t* dNums, const uint16_t* dExp, unsigned R, unsigned nIn, uint16_t* dCoeff,
                const GfTables& gt, cudaStream_t st)
{
	const size_t n = (size_t)R * nIn;
	if(!n) return 0;
	k_par2_coeffs<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(dNums, dExp, R, nIn, dCoeff, gt);
	P2C_CUDA_TRY(cudaGetLastError());
	return 0;
}

// coefficient matrix [R][nIn] -> index layout (used by the device-level entry point)
__global__ void k_coeff_to_idx(const uint16_t* coeff, unsigned R, unsigned nIn, unsigned G, uint4* idx)
{
	const size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
	if(id >= (size_t)R * G) return;
	const unsigned r = (unsigned)(id / G), g = (unsigned)(id % G);
	uint32_t q[4] = {0, 0, 0, 0};
#pragma unroll
	for(int t = 0; t < 8; t++) {
		unsigned i = g * 8 + t;
		uint32_t c = i < nIn ? coeff[(size_t)r * nIn + i] : 0;
#pragma unroll
		for(int k = 0; k < 16; k++) q[k >> 2] |= ((c >> k) & 1u) << (8 * (k & 3) + t);
	}
	idx[(size_t)r * G + g] = make_uint4(q[0], q[1], q[2], q[3]);
}

int coeff_to_idx(const uint16_t* dCoeff, unsigned R, unsigned nIn, uint4* dIdx, cudaStream_t st)
{
	unsigned G = (nIn + 7) / 8;
	size_t n = (size_t)R * G;
	if(!n) return 0;
	k_coeff_to_idx<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(dCoeff, R, nIn, G, dIdx);
	P2C_CUDA_TRY(cudaGetLastError());
	return 0;
}

// ---- seeded synthetic data (same bytes as parpar_gb300/synth.py) -------------
__device__ __forceinline__ uint64_t splitmix_mix(uint64_t z) {
	z ^= z >> 30; z *= 0xBF58476D1CE4E5B9ull;
	z ^= z >> 27; z *= 0x94D049BB133111EBull;
	return z ^ (z >> 31);
}
__global__ void k_synth(uint8_t* dst, size_t pitchBytes, unsigned nRows, size_t rowBytes, uint64_t seed, uint64_t first,
                        uint64_t unitOffset)
{
	const size_t units = (rowBytes + 7) / 8;
	const size_t total = units * nRows;
	for(size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x; id < total; id += (size_t)gridDim.x * blockDim.x) {
		size_t row = id / units, u = id % units;
		uint64_t z = splitmix_mix(seed * 0xD1342543DE82EF95ull + (first + row) * 0x9E3779B97F4A7C15ull + unitOffset + u);
		uint8_t* p = dst + row * pitchBytes + u * 8;
		if(u * 8 + 8 <= rowBytes && ((reinterpret_cast<uintptr_t>(p) & 7) == 0)) {
			*reinterpret_cast<uint64_t*>(p) = z;
		} else {
			for(size_t b = 0; b < 8 && u * 8 + b < rowBytes; b++) p[b] = (uint8_t)(z >> (8 * b));
		}
	}
}

int synth_fill(void* dst, size_t pitchBytes, unsigned nRows, size_t rowBytes, uint64_t seed, uint64_t first, cudaStream_t st,
               uint64_t byteOffset)
{
	if(byteOffset % 8) { set_error("synthetic window offset must be a multiple of 8"); return -1; }
	size_t total = (rowBytes + 7) / 8 * (size_t)nRows;
	if(!total) return 0;
	unsigned blocks = (unsigned)std::min<size_t>((total + 255) / 256, 152 * 32);
	k_synth<<<blocks, 256, 0, st>>>((uint8_t*)dst, pitchBytes, nRows, rowBytes, seed, first, byteOffset / 8);
	P2C_CUDA_TRY(cudaGetLastError());
	return 0;
}

} // namespace p2c
