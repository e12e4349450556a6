// Tensor-core (tcgen05) variant of the multiply-accumulate: the GF(2^16)
// contraction written as a dense GF(2) matrix product on the 5th-generation
// tensor cores, parity taken from the accumulator.
//
//   A[16r + j][16i + b] = bit j of (c(r,i) * x^b)   (the 16x16 bit matrix of c)
//   B[16i + b][w]       = bit b of in_i[w]           (input bit planes)
//   C[16r + j][w]       = sum_{i,b} A * B  (an integer <= 16 * nIn)
//   bit j of rec_r[w]   = C[16r + j][w] & 1
//
// Operands are 0/1 values in e4m3 (1.0 = 0x38) for kind::f8f6f4 with fp32
// accumulators, exact below 2^24 = 16 * 2^20 inputs.  (ptxas rejects
// tcgen05.mma .kind::i8 for sm_103a: GB300 has no int8 MMA, so the int32-
// accumulator form of this product is not available on this GPU; the
// template keeps the integer path for targets that have it.)
// Both are expanded from the compact data on the fly into shared memory in
// the K-major 128-byte-swizzled layout (8-row x 128-byte atoms, 16-byte chunk
// q of row m stored at chunk q ^ (m & 7)); one K stage = 8 inputs x 16 bits =
// 128 bytes per row.
//
// CTA: 16 recovery slices (two M = 128 accumulators, 8 slices x 16 bit rows
// each) x 256 words (N = 256), all inputs.  Warp 0 allocates the 512 TMEM
// columns and one thread issues the MMAs (4 x K = 32 per accumulator per
// stage) and commits to the stage's "empty" mbarrier; warps 1-11 expand the
// next stages (3-stage ring, "full" mbarriers).  Epilogue: each warp reads its
// 32 TMEM lanes with tcgen05.ld, takes the parity bits and packs 16 bit rows
// into words with a warp ballot.  Every wait is bounded (error flag, no hang).
#include "common.cuh"
#include "kernels.h"

namespace p2c {

#define TC_BN 256
#define TC_SLICES 16
#define TC_NST 3
#define TC_STAGE 65536
#define TC_PRODUCERS 352   /* warps 1..11 */
#define TC_THREADS 384
#define TC_BQ 1           /* B items (256) per producer, rounded up */
#define TC_AQ 6           /* A items (2048) per producer, rounded up */
#define TC_WAIT_LIMIT (1u << 24)

__device__ unsigned g_tc_error;

__device__ __forceinline__ unsigned tc_saddr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void tc_bar_init(uint32_t a, unsigned count) {
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(a), "r"(count) : "memory");
}
__device__ __forceinline__ void tc_bar_arrive(uint32_t a) {
	asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" :: "r"(a) : "memory");
}
__device__ __forceinline__ bool tc_bar_wait(uint32_t a, unsigned parity) {
	for(unsigned i = 0; i < TC_WAIT_LIMIT; i++) {
		unsigned ok;
		asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
		             : "=r"(ok) : "r"(a), "r"(parity) : "memory");
		if(ok) return true;
	}
	atomicExch(&g_tc_error, 1u);
	return false;
}

// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr) {
	uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
	d |= (uint64_t)1 << 16;             // leading byte offset (unused for swizzled K-major)
	d |= (uint64_t)(1024 >> 4) << 32;   // stride byte offset
	d |= (uint64_t)1 << 46;             // descriptor version
	d |= (uint64_t)2 << 61;             // 128-byte swizzle
	return d;
}

// instruction descriptor: M = 128, N = 256, K-major A and B; i8: unsigned
// 8-bit operands, s32 accumulators; fp8: e4m3 operands, f32 accumulators
template<bool FP8> __device__ __forceinline__ uint32_t tc_idesc() {
	return (FP8 ? (1u << 4) : (2u << 4)) | ((uint32_t)(TC_BN >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

template<bool FP8>
__device__ __forceinline__ void tc_mma(uint32_t dTmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accum) {
	static_assert(FP8, "sm_103a has no integer tcgen05 MMA");
	asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
	             "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}"
	             :: "r"(dTmem), "l"(a), "l"(b), "r"(idesc), "r"(accum) : "memory");
}

__device__ __forceinline__ void tc_ld32(uint32_t taddr, uint32_t (&v)[32]) {
	asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 "
	             "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
	             "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
	             : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
	               "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
	               "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
	               "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
	             : "r"(taddr));
	asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// 16 bits -> 16 bytes (byte b = bit b of x times `one`)
__device__ __forceinline__ uint4 tc_expand16(uint32_t x, uint32_t one) {
	uint32_t o[4];
#pragma unroll
	for(int q = 0; q < 4; q++) {
		const uint32_t t = (x >> (4 * q)) & 15u;
		o[q] = ((t * 0x00204081u) & 0x01010101u) * one;
	}
	return make_uint4(o[0], o[1], o[2], o[3]);
}

// in-register 16x16 bit transpose: out[j] bit b = in[b] bit j
__device__ __forceinline__ void tc_transpose16(uint32_t (&m)[16]) {
#pragma unroll
	for(int k = 0; k < 8; k++) { uint32_t t = ((m[k] >> 8) ^ m[k + 8]) & 0x00FFu; m[k] ^= t << 8; m[k + 8] ^= t; }
#pragma unroll
	for(int k = 0; k < 16; k++) if((k & 4) == 0 && k < 12) { uint32_t t = ((m[k] >> 4) ^ m[k + 4]) & 0x0F0Fu; m[k] ^= t << 4; m[k + 4] ^= t; }
#pragma unroll
	for(int k = 0; k < 16; k++) if((k & 2) == 0 && k < 14) { uint32_t t = ((m[k] >> 2) ^ m[k + 2]) & 0x3333u; m[k] ^= t << 2; m[k + 2] ^= t; }
#pragma unroll
	for(int k = 0; k < 16; k += 2) { uint32_t t = ((m[k] >> 1) ^ m[k + 1]) & 0x5555u; m[k] ^= t << 1; m[k + 1] ^= t; }
}

// Row masks of every coefficient's bit matrix, once per launch: rows[r][i][j]
// = sum_b bit_j(c(r,i) * x^b) << b (so a CTA does not redo the 16-step
// multiply chain and the bit transpose for every word tile).
__global__ void k_tc_rows(const uint16_t* __restrict__ coeff, unsigned R, unsigned nIn, uint4* __restrict__ rows)
{
	const size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
	if(id >= (size_t)R * nIn) return;
	uint32_t m[16];
	m[0] = coeff[id];
#pragma unroll
	for(int b = 1; b < 16; b++) {
		const uint32_t v = m[b - 1] << 1;
		m[b] = (v ^ ((v >> 16) * (P2C_POLY & 0xFFFFu))) & 0xFFFFu;
	}
	tc_transpose16(m);
	rows[id * 2] = make_uint4(m[0] | (m[1] << 16), m[2] | (m[3] << 16), m[4] | (m[5] << 16), m[6] | (m[7] << 16));
	rows[id * 2 + 1] = make_uint4(m[8] | (m[9] << 16), m[10] | (m[11] << 16), m[12] | (m[13] << 16), m[14] | (m[15] << 16));
}

template<bool FP8>
__global__ void __launch_bounds__(TC_THREADS, 1) k_tc_muladd(
	const uint16_t* __restrict__ in, size_t inPitch, unsigned nIn,
	const uint16_t* __restrict__ maskRows, uint16_t* __restrict__ rec, size_t recPitch, unsigned R, size_t nWords,
	int accumulate)
{
	extern __shared__ __align__(1024) uint8_t smem_raw[];
	const uint32_t raw = tc_saddr(smem_raw);
	const uint32_t pad = (1024u - (raw & 1023u)) & 1023u;
	uint8_t* sm = smem_raw + pad;
	const uint32_t sbase = raw + pad;
	const uint32_t barBase = sbase + TC_NST * TC_STAGE;     // full[NST], empty[NST], done
	uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + TC_NST * TC_STAGE + (2 * TC_NST + 1) * 8);
	auto fullBar = [&](int s) { return barBase + 8u * s; };
	auto emptyBar = [&](int s) { return barBase + 8u * (TC_NST + s); };
	const uint32_t doneBar = barBase + 8u * (2 * TC_NST);

	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const size_t colBase = (size_t)blockIdx.x * TC_BN;
	const unsigned rbase = blockIdx.y * TC_SLICES;
	const unsigned G = (nIn + 7) / 8;
	const uint32_t one = FP8 ? 0x38u : 1u;

	if(threadIdx.x == 0) {
		for(int s = 0; s < TC_NST; s++) {
			tc_bar_init(fullBar(s), TC_PRODUCERS);
			tc_bar_init(emptyBar(s), 1);
		}
		tc_bar_init(doneBar, 1);
	}
	if(warp == 0) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" :: "r"(tc_saddr(tslot)), "r"(512u) : "memory");
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
	}
	asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
	__syncthreads();
	asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
	const uint32_t tmem = *tslot;

	if(warp == 0) {
		if(lane == 0) {
			const uint32_t idesc = tc_idesc<FP8>();
			for(unsigned g = 0; g < G; g++) {
				const int s = g % TC_NST;
				if(!tc_bar_wait(fullBar(s), (g / TC_NST) & 1)) break;
				asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
				const uint32_t st = sbase + s * TC_STAGE;
#pragma unroll
				for(int a = 0; a < 2; a++)
#pragma unroll
					for(int k = 0; k < 4; k++)
						tc_mma<FP8>(tmem + a * 256, tc_desc(st + a * 16384 + k * 32), tc_desc(st + 32768 + k * 32), idesc,
						            (g | k) != 0);
				asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" :: "r"(emptyBar(s)) : "memory");
			}
			asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" :: "r"(doneBar) : "memory");
		}
		__syncwarp();
	} else {
		// producers: expand stage g's B (input bit planes, 256 items of 8 words)
		// and A (coefficient bit-matrix rows, 2048 items of one row).  The
		// global loads of stage g+1 are issued before stage g is expanded, so
		// their latency overlaps the expansion.
		const int pt = threadIdx.x - 32;
		uint4 bv[TC_BQ], bvN[TC_BQ];
		uint32_t am[TC_AQ], amN[TC_AQ];
		auto load_stage = [&](unsigned g, uint4 (&b)[TC_BQ], uint32_t (&am_)[TC_AQ]) {
#pragma unroll
			for(int q = 0; q < TC_BQ; q++) {
				const int item = pt + q * TC_PRODUCERS;
				b[q] = make_uint4(0, 0, 0, 0);
				if(item < 256) {
					const int t = item >> 5, w8 = item & 31;
					const unsigned i = g * 8 + t;
					const size_t col = colBase + w8 * 8;
					if(i < nIn && col < nWords) {
						const uint16_t* src = in + (size_t)i * inPitch + col;
						if(col + 8 <= nWords) b[q] = __ldg(reinterpret_cast<const uint4*>(src));
						else {
							uint32_t tmp[4] = {0, 0, 0, 0};
							for(size_t c = col; c < nWords; c++) tmp[(c - col) >> 1] |= (uint32_t)__ldg(src + (c - col)) << (16 * ((c - col) & 1));
							b[q] = make_uint4(tmp[0], tmp[1], tmp[2], tmp[3]);
						}
					}
				}
			}
#pragma unroll
			for(int q = 0; q < TC_AQ; q++) {
				const int it = pt + q * TC_PRODUCERS;
				am_[q] = 0;
				if(it < 2048) {
					const int j = it & 15, t = (it >> 4) & 7, sl = (it >> 7) & 7, a = it >> 10;
					const unsigned r = rbase + a * 8 + sl, i = g * 8 + t;
					if(r < R && i < nIn) am_[q] = __ldg(maskRows + ((size_t)r * nIn + i) * 16 + j);
				}
			}
		};
		if(G) load_stage(0, bv, am);
		for(unsigned g = 0; g < G; g++) {
			const int s = g % TC_NST;
			const unsigned use = g / TC_NST;
			if(g + 1 < G) load_stage(g + 1, bvN, amN);
			if(use > 0 && !tc_bar_wait(emptyBar(s), (use - 1) & 1)) break;
			uint8_t* st = sm + s * TC_STAGE;
#pragma unroll
			for(int q = 0; q < TC_BQ; q++) {
				const int item = pt + q * TC_PRODUCERS;
				if(item >= 256) continue;
				const int t = item >> 5, w0 = (item & 31) * 8;
				const uint32_t wv[4] = {bv[q].x, bv[q].y, bv[q].z, bv[q].w};
#pragma unroll
				for(int e = 0; e < 8; e++) {
					const int w = w0 + e;
					const uint32_t x = (wv[e >> 1] >> (16 * (e & 1))) & 0xFFFFu;
					*reinterpret_cast<uint4*>(st + 32768 + w * 128 + ((t ^ (w & 7)) << 4)) = tc_expand16(x, one);
				}
			}
#pragma unroll
			for(int q = 0; q < TC_AQ; q++) {
				const int it = pt + q * TC_PRODUCERS;
				if(it < 2048) {
					const int j = it & 15, t = (it >> 4) & 7, sl = (it >> 7) & 7, a = it >> 10;
					const int m = sl * 16 + j;
					*reinterpret_cast<uint4*>(st + a * 16384 + m * 128 + ((t ^ (m & 7)) << 4)) = tc_expand16(am[q], one);
				}
			}
			asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
			tc_bar_arrive(fullBar(s));
#pragma unroll
			for(int q = 0; q < TC_BQ; q++) bv[q] = bvN[q];
#pragma unroll
			for(int q = 0; q < TC_AQ; q++) am[q] = amN[q];
		}
	}

	// epilogue: parity of every accumulator element, 16 bit rows -> one word
	const bool ok = tc_bar_wait(doneBar, 0);
	asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
	if(ok && warp < 8) {   // warps 0-3: accumulator 0, warps 4-7: accumulator 1
		const int a = warp >> 2, wq = warp & 3;
		const unsigned r0 = rbase + a * 8 + 2 * wq;
		for(int cc = 0; cc < TC_BN / 32; cc++) {
			uint32_t v[32];
			tc_ld32(tmem + ((uint32_t)(32 * wq) << 16) + a * 256 + cc * 32, v);
			uint32_t mine = 0;
#pragma unroll
			for(int c = 0; c < 32; c++) {
				const uint32_t par = FP8 ? (__float2uint_rz(__uint_as_float(v[c])) & 1u) : (v[c] & 1u);
				const uint32_t bal = __ballot_sync(0xFFFFFFFFu, par);
				if(lane == c) mine = bal;
			}
			const size_t col = colBase + cc * 32 + lane;
			if(col < nWords) {
				if(r0 < R) {
					uint16_t* p = rec + (size_t)r0 * recPitch + col;
					uint16_t val = (uint16_t)(mine & 0xFFFFu);
					*p = accumulate ? (uint16_t)(*p ^ val) : val;
				}
				if(r0 + 1 < R) {
					uint16_t* p = rec + (size_t)(r0 + 1) * recPitch + col;
					uint16_t val = (uint16_t)(mine >> 16);
					*p = accumulate ? (uint16_t)(*p ^ val) : val;
				}
			}
		}
	}
	asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
	__syncthreads();
	if(warp == 0)
		asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(512u) : "memory");
}

size_t tc_scratch_bytes(unsigned R, unsigned nIn) { return (size_t)R * nIn * 32; }

int tc_muladd(const uint16_t* in, size_t inPitch, unsigned nIn, const uint16_t* coeff, uint16_t* rec, size_t recPitch,
              unsigned R, size_t nWords, int accumulate, bool fp8, void* scratch, size_t scratchBytes, cudaStream_t st)
{
	if(!R || !nWords) return 0;
	if(scratchBytes < tc_scratch_bytes(R, nIn) || (!scratch && nIn)) {
		set_error("tensor method needs %zu bytes of scratch, %zu given", tc_scratch_bytes(R, nIn), scratchBytes);
		return -1;
	}
	if(!nIn) {
		if(!accumulate) P2C_CUDA_TRY(cudaMemset2DAsync(rec, recPitch * 2, 0, nWords * 2, R, st));
		return 0;
	}
	const size_t smem = TC_NST * TC_STAGE + (2 * TC_NST + 1) * 8 + 16 + 1024;
	dim3 grid((unsigned)((nWords + TC_BN - 1) / TC_BN), (R + TC_SLICES - 1) / TC_SLICES);
	if(!fp8) { set_error("integer tensor-core MMA is not available on sm_103a"); return -1; }
	const size_t nc = (size_t)R * nIn;
	k_tc_rows<<<(unsigned)((nc + 255) / 256), 256, 0, st>>>(coeff, R, nIn, reinterpret_cast<uint4*>(scratch));
	P2C_CUDA_TRY(cudaGetLastError());
	P2C_CUDA_TRY(cudaFuncSetAttribute(k_tc_muladd<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
	k_tc_muladd<true><<<grid, TC_THREADS, smem, st>>>(in, inPitch, nIn, reinterpret_cast<const uint16_t*>(scratch), rec, recPitch,
	                                           R, nWords, accumulate);
	P2C_CUDA_TRY(cudaGetLastError());
	return 0;
}

int tc_error_take() {
	unsigned v = 0, z = 0;
	if(cudaMemcpyFromSymbol(&v, g_tc_error, sizeof(v)) != cudaSuccess) return -1;
	if(v) cudaMemcpyToSymbol(g_tc_error, &z, sizeof(z));
	return (int)v;
}

} // namespace p2c
