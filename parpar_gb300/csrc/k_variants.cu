// Two further multiply-accumulate variants with the comb kernel's contract
// (rec[r] (^)= sum_i c(r,i) in[i] over nWords words), kept for comparison and
// for the autotuner:
//
//  * xor    — the LOP3 formulation of the reference's XOR bit-dependency method
//             (gf16/gf16_xor_*.c, xor_depends/info.md): multiplication by c is
//             split over the 16 bits of c, P[k] ^= in & -(bit k of c), i.e. one
//             3-input LOP3 per (coefficient bit, 32-bit word pair), and the 16
//             partial sums are folded by Horner (x^k) at the end.  No tables,
//             no shared memory: bound by the integer pipe (~8 LOP3 per word
//             mul-add plus mask generation).
//  * nibble — split-nibble tables (the OpenCL LOOKUP idea,
//             gf16/controller_ocl_init.cpp:112-253, with 4 x 16-entry tables per
//             coefficient instead of 2 x 256): c*x = T0[x&15]^T1[x>>4&15]^
//             T2[x>>8&15]^T3[x>>12], tables built per CTA in shared memory.
#include "common.cuh"
#include "kernels.h"

namespace p2c {

// ------------------------------------------------------------------ xor (LOP3)
// CTA: 8 warps; warp w handles recovery row blockIdx.y*8 + w; each lane owns
// 8 consecutive u32 (16 words) of the CTA's 512-word tile.
__global__ void __launch_bounds__(256) k_xor_muladd(
	const uint16_t* __restrict__ in, size_t inPitch, unsigned nIn, const uint16_t* __restrict__ coeff,
	uint16_t* __restrict__ rec, size_t recPitch, unsigned R, size_t nWords, int accumulate)
{
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const unsigned r = blockIdx.y * 8 + warp;
	if(r >= R) return;
	const size_t w0 = (size_t)blockIdx.x * 512 + lane * 16;
	if(w0 >= nWords) return;
	uint32_t P[16][8];
#pragma unroll
	for(int k = 0; k < 16; k++)
#pragma unroll
		for(int v = 0; v < 8; v++) P[k][v] = 0;
	const uint16_t* crow = coeff + (size_t)r * nIn;
	for(unsigned i = 0; i < nIn; i++) {
		const uint32_t c = __ldg(crow + i);
		const uint4* src = reinterpret_cast<const uint4*>(in + (size_t)i * inPitch + w0);
		const uint4 a = __ldg(src), b = __ldg(src + 1);
		const uint32_t d[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
		for(int k = 0; k < 16; k++) {
			const uint32_t m = 0u - ((c >> k) & 1u);
#pragma unroll
			for(int v = 0; v < 8; v++) P[k][v] ^= d[v] & m;  // one LOP3
		}
	}
	uint32_t* dst = reinterpret_cast<uint32_t*>(rec + (size_t)r * recPitch + w0);
#pragma unroll
	for(int v = 0; v < 8; v++) {
		uint32_t acc = P[15][v];
#pragma unroll
		for(int k = 14; k >= 0; k--) acc = mul2x2(acc) ^ P[k][v];
		if(accumulate) acc ^= dst[v];
		dst[v] = acc;
	}
}

int xor_muladd(const uint16_t* in, size_t inPitch, unsigned nIn, const uint16_t* coeff, uint16_t* rec,
               size_t recPitch, unsigned R, size_t nWords, int accumulate, cudaStream_t st)
{
	if(!R || !nWords) return 0;
	// tiles of 512 words; rows are padded to 64-word multiples, so round the
	// tile count down to what the pitch holds and require 16-word alignment
	size_t nw = round_up(nWords, 16);
	dim3 grid((unsigned)((nw + 511) / 512), (R + 7) / 8);
	k_xor_muladd<<<grid, 256, 0, st>>>(in, inPitch, nIn, coeff, rec, recPitch, R, nw, accumulate);
	P2C_CUDA_TRY(cudaGetLastError());
	return 0;
}

// ------------------------------------------------------------ nibble tables
// CTA: 256 threads, tile of 512 words (one u32 = 2 words per thread), 8
// recovery rows; inputs are consumed 4 at a time with 8x4 coefficient tables
// of 4 x 16 u16 entries in shared memory.
__global__ void __launch_bounds__(256) k_nibble_muladd(
	const uint16_t* __restrict__ in, size_t inPitch, unsigned nIn, const uint16_t* __restrict__ coeff,
	uint16_t* __restrict__ rec, size_t recPitch, unsigned R, size_t nWords, int accumulate, GfTables gt)
{
	__shared__ uint16_t tab[8][4][64]; // [row][input in step][nibble pos * 16 + value]
	const unsigned rbase = blockIdx.y * 8;
	const size_t w = (size_t)blockIdx.x * 512 + threadIdx.x * 2;
	const bool active = w < nWords;
	uint32_t acc[8];
#pragma unroll
	for(int s = 0; s < 8; s++) acc[s] = 0;
	const uint32_t* in32 = reinterpret_cast<const uint32_t*>(in);
	for(unsigned i0 = 0; i0 < nIn; i0 += 4) {
		__syncthreads();
		// build: 8 rows x 4 inputs x 64 entries = 2048 entries, 8 per thread
		for(int e = threadIdx.x; e < 2048; e += 256) {
			const int s = e >> 8, t = (e >> 6) & 3, q = (e >> 4) & 3, v = e & 15;
			const unsigned r = rbase + s, i = i0 + t;
			uint16_t c = (r < R && i < nIn) ? __ldg(coeff + (size_t)r * nIn + i) : 0;
			tab[s][t][q * 16 + v] = gf_mul_tab(gt, c, (uint16_t)(v << (4 * q)));
		}
		__syncthreads();
		if(!active) continue;
#pragma unroll
		for(int t = 0; t < 4; t++) {
			const unsigned i = i0 + t;
			const uint32_t x = i < nIn ? __ldg(in32 + ((size_t)i * inPitch + w) / 2) : 0u;
#pragma unroll
			for(int s = 0; s < 8; s++) {
				const uint16_t* T = tab[s][t];
				uint32_t lo = T[x & 15] ^ T[16 + (x >> 4 & 15)] ^ T[32 + (x >> 8 & 15)] ^ T[48 + (x >> 12 & 15)];
				uint32_t hi = T[x >> 16 & 15] ^ T[16 + (x >> 20 & 15)] ^ T[32 + (x >> 24 & 15)] ^ T[48 + (x >> 28)];
				acc[s] ^= lo | (hi << 16);
			}
		}
	}
	if(!active) return;
	uint32_t* rec32 = reinterpret_cast<uint32_t*>(rec);
#pragma unroll
	for(int s = 0; s < 8; s++) {
		const unsigned r = rbase + s;
		if(r < R) {
			uint32_t* p = rec32 + ((size_t)r * recPitch + w) / 2;
			*p = accumulate ? (*p ^ acc[s]) : acc[s];
		}
	}
}

int nibble_muladd_t(const uint16_t* in, size_t inPitch, unsigned nIn, const uint16_t* coeff, uint16_t* rec,
                    size_t recPitch, unsigned R, size_t nWords, int accumulate, const GfTables& gt, cudaStream_t st)
{
	if(!R || !nWords) return 0;
	size_t nw = round_up(nWords, 2);
	dim3 grid((unsigned)((nw + 511) / 512), (R + 7) / 8);
	k_nibble_muladd<<<grid, 256, 0, st>>>(in, inPitch, nIn, coeff, rec, recPitch, R, nw, accumulate, gt);
	P2C_CUDA_TRY(cudaGetLastError());
	return 0;
}

} // namespace p2c
