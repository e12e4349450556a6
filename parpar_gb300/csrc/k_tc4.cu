// The GF(2^16) contraction as a block-scaled 4-bit matrix product on tcgen05
// (kind::mxf4), with both operands loaded by TMA.
//
//   D[w][16r + j] = sum_{i,b} A[w][16i + b] * B[16r + j][16i + b]
//   A[w][16i + b] = bit b of in_i[w]                    (input bit planes)
//   B[16r+j][16i+b] = bit j of (c(r,i) * x^b)           (the 16x16 GF(2) matrix of c)
//   bit j of rec_r[w] = D[w][16r + j] mod 2
//
// Operands are e2m1 values 0 and 1.0 (nibble 0x2), two per byte, K-major;
// their block scale factors are all 1.0 (ue8m0 0x7F), so every product is
// exactly 0 or 1 and the fp32 accumulators hold exact integers (< 2^24 for
// fewer than 2^20 inputs).  Both operands are expanded once per call into
// scratch in HBM by two preparation kernels: the inputs 4x (k_tc4_prep_in: a
// word chunk of the inputs at a time), the coefficient matrix to its bit rows
// (k_tc4_prep_coeff).
//
// GEMM: persistent, one CTA of 192 threads per SM taking 128-word x
// 256-bit-row tiles (16 recovery slices, all K) from a global tile counter,
// in raster order, so that a CTA that starts late (its SM held by another
// kernel) simply takes fewer tiles.  Thread 0 issues the TMA loads of a
// 4-stage ring (A: 128 rows x 128 bytes, B: 256 rows x 128 bytes, 128-byte
// swizzle) completing on "full" mbarriers, across tile boundaries, and
// publishes each tile number to the other roles; thread 32 issues 4 MMAs
// (M=128, N=256, K=64) per stage into the TMEM accumulator (columns 0-255;
// the scale factors, all 1.0, in columns 448-511) and commits each stage to
// its "empty" mbarrier and each tile to "tmemFull"; warps 2-5 read the
// accumulator with tcgen05.ld (each thread one word and 256 columns, i.e. 16
// recovery words, whose bits are the accumulators' parities) and release it.
// A second tile shape (192 rows, two accumulators) can be selected.  Tiles
// are grouped by word tiles (as many as keep their A tiles in about 48 MiB of
// L2) that walk the recovery tiles together, so A is read from HBM once and
// each B tile once per group.
// Every wait is bounded (error flag g_tc4_error, no hang).
#include "common.cuh"
#include "kernels.h"

#include <cuda.h>   // CUtensorMap and its enums (types only; the encoder comes from the runtime)

#include <atomic>

namespace p2c {

#define T4_BM 128
#define T4_KB 128
#define T4_TR 8           // ring of published tile numbers
#define T4_NO_TILE 0xFFFFFFFFu
#define T4_ACC_STRIDE 256 // TMEM columns between the two accumulators
#define T4_SFA_COL 448    // TMEM columns of the scale factors (A, then B)
#define T4_SFB_COL 480
#define T4_STAGE_A (T4_BM * T4_KB)
#define T4_RCOMMON 48     // recovery padding of B: a multiple of both tiles' slice counts

// The two tile shapes: 256 bit rows (16 recovery slices) with one TMEM
// accumulator and a 4-stage ring (the default), or 192 bit rows (12 slices)
// with two accumulators (the next tile's MMAs overlap the read-out) and a
// 5-stage ring (selectable; measured slower, see tc4_shape_for).
template<int BN> struct T4Shape {
	static constexpr int RPT = BN / 16;
	static constexpr int NACC = BN <= 192 ? 2 : 1;
	static constexpr int NST = BN <= 192 ? 5 : 4;
	static constexpr int STAGE = T4_STAGE_A + BN * T4_KB;
	// mbarriers after the stages
	static constexpr int BAR_FULL = 0;                  // [NST] a stage's operands landed
	static constexpr int BAR_EMPTY = NST;               // [NST] a stage's MMAs completed
	static constexpr int BAR_TFULL = 2 * NST;           // [2] an accumulator holds a finished tile
	static constexpr int BAR_TEMPTY = 2 * NST + 2;      // [2] the epilogue has read it (4 arrivals)
	static constexpr int BAR_IDFULL = 2 * NST + 4;      // [TR] a tile number was published
	static constexpr int BAR_IDEMPTY = BAR_IDFULL + T4_TR; // [TR] its readers have read it (5 arrivals)
	static constexpr int BAR_DRAIN = BAR_IDEMPTY + T4_TR;
	static constexpr int NBARS = BAR_DRAIN + 1;
	static constexpr size_t SMEM = (size_t)NST * STAGE + NBARS * 8 + (T4_TR + 2) * 4 + 1024;
	static_assert(NACC == 1 || T4_ACC_STRIDE + BN <= T4_SFA_COL, "accumulators overlap the scale factors");
	static_assert(BN <= T4_SFA_COL, "accumulator overlaps the scale factors");
	static_assert(SMEM <= 227 * 1024, "shared memory");
};
#define T4_WAIT (1u << 24)
#define T4_THREADS 192
#define T4_A_CHUNK_BYTES (1ull << 30)

__device__ unsigned g_tc4_error;

// ------------------------------------------------------------------ operands
// 4 bits -> 4 nibbles holding e2m1 1.0 (0x2) where the bit is set
__device__ __forceinline__ uint32_t t4_spread4(uint32_t t) {
	return ((t | (t << 3) | (t << 6) | (t << 9)) & 0x1111u) << 1;
}
// 16 bits -> 8 bytes, bit k in nibble k (element 2h in the low nibble of byte h)
__device__ __forceinline__ uint2 t4_spread16(uint32_t x) {
	return make_uint2(t4_spread4(x & 15u) | (t4_spread4((x >> 4) & 15u) << 16),
	                  t4_spread4((x >> 8) & 15u) | (t4_spread4((x >> 12) & 15u) << 16));
}

// A chunk: rows w = w0 .. w0 + rows-1 (zero past nWords), 8 bytes per input
// (zero for inputs >= nIn up to kBytes / 8).  Block: 64 inputs x 64 words.
__global__ void __launch_bounds__(256) k_tc4_prep_in(const uint16_t* __restrict__ in, size_t inPitch, unsigned nIn,
                                                   size_t nWords, size_t w0, uint8_t* __restrict__ A, size_t kBytes)
{
	__shared__ uint16_t tile[64][65];
	const unsigned i0 = blockIdx.y * 64;
	const size_t wt = w0 + (size_t)blockIdx.x * 64;
	for(int e = threadIdx.x; e < 64 * 64; e += 256) {
		const int ii = e >> 6, ww = e & 63;
		const unsigned i = i0 + ii;
		const size_t w = wt + ww;
		tile[ii][ww] = (i < nIn && w < nWords) ? __ldg(in + (size_t)i * inPitch + w) : (uint16_t)0;
	}
	__syncthreads();
	const int ii = threadIdx.x & 63;
	if((size_t)(i0 + ii) * 8 >= kBytes) return;
	for(int ww = threadIdx.x >> 6; ww < 64; ww += 4) {
		const uint2 v = t4_spread16(tile[ii][ww]);
		*reinterpret_cast<uint2*>(A + ((size_t)blockIdx.x * 64 + ww) * kBytes + (size_t)(i0 + ii) * 8) = v;
	}
}

// The same with 16-byte loads and stores, for inputs whose base and pitch are
// 16-byte aligned.  Block: 64 inputs x 128 words; thread t loads 8-word
// segments (t & 15) of rows t / 16 + 16k, and writes, for the input pair
// 2 (t & 31), 2 (t & 31) + 1, the 16 bytes of words t / 32 + 8k.  A segment is
// loaded only when its first word is below nWords (rows are readable up to
// roundup(nWords, 64) words); words past nWords are zero.
__global__ void __launch_bounds__(256) k_tc4_prep_in_v(const uint16_t* __restrict__ in, size_t inPitch, unsigned nIn,
                                                     size_t nWords, size_t w0, uint8_t* __restrict__ A, size_t kBytes)
{
	__shared__ uint16_t tile[64][130];
	const unsigned i0 = blockIdx.y * 64;
	const size_t wt = w0 + (size_t)blockIdx.x * 128;
	const unsigned t = threadIdx.x;
#pragma unroll
	for(int k = 0; k < 4; k++) {
		const unsigned ii = (t >> 4) + 16 * k, seg = t & 15;
		const unsigned i = i0 + ii;
		const size_t w = wt + 8 * seg;
		uint4 v = make_uint4(0, 0, 0, 0);
		if(i < nIn && w < nWords) {
			v = __ldg(reinterpret_cast<const uint4*>(in + (size_t)i * inPitch + w));
			const size_t valid = nWords - w;
			if(valid < 8) {
				uint32_t* e = reinterpret_cast<uint32_t*>(&v);
#pragma unroll
				for(int q = 0; q < 4; q++) {
					if((size_t)(2 * q) >= valid) e[q] = 0;
					else if((size_t)(2 * q + 1) >= valid) e[q] &= 0xFFFFu;
				}
			}
		}
		uint32_t* row = reinterpret_cast<uint32_t*>(&tile[ii][8 * seg]);
		row[0] = v.x; row[1] = v.y; row[2] = v.z; row[3] = v.w;
	}
	__syncthreads();
	const unsigned ip = t & 31;
	if((size_t)(i0 + 2 * ip) * 8 >= kBytes) return;
#pragma unroll 4
	for(unsigned ww = t >> 5; ww < 128; ww += 8) {
		const uint2 a = t4_spread16(tile[2 * ip][ww]), b = t4_spread16(tile[2 * ip + 1][ww]);
		*reinterpret_cast<uint4*>(A + ((size_t)blockIdx.x * 128 + ww) * kBytes + (size_t)(i0 + 2 * ip) * 8) =
			make_uint4(a.x, a.y, b.x, b.y);
	}
}

// B: rows 16r + j for r < rPad (zero rows past R), 8 bytes per input; one
// thread per (r, i).
__global__ void __launch_bounds__(256) k_tc4_prep_coeff(const uint16_t* __restrict__ coeff, unsigned R, unsigned nIn,
                                                      unsigned rPad, unsigned nInPad, uint8_t* __restrict__ B)
{
	const size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
	if(id >= (size_t)rPad * nInPad) return;
	const unsigned r = (unsigned)(id / nInPad), i = (unsigned)(id % nInPad);
	uint32_t m[16];
	m[0] = (r < R && i < nIn) ? __ldg(coeff + (size_t)r * nIn + i) : 0u;
#pragma unroll
	for(int b = 1; b < 16; b++) {
		const uint32_t v = m[b - 1] << 1;
		m[b] = (v ^ ((v >> 16) * (P2C_POLY & 0xFFFFu))) & 0xFFFFu;
	}
	// transpose: rows[j] bit b = bit j of c * x^b
#pragma unroll
	for(int k = 0; k < 8; k++) { uint32_t t = ((m[k] >> 8) ^ m[k + 8]) & 0x00FFu; m[k] ^= t << 8; m[k + 8] ^= t; }
#pragma unroll
	for(int k = 0; k < 16; k++) if((k & 4) == 0 && k < 12) { uint32_t t = ((m[k] >> 4) ^ m[k + 4]) & 0x0F0Fu; m[k] ^= t << 4; m[k + 4] ^= t; }
#pragma unroll
	for(int k = 0; k < 16; k++) if((k & 2) == 0 && k < 14) { uint32_t t = ((m[k] >> 2) ^ m[k + 2]) & 0x3333u; m[k] ^= t << 2; m[k + 2] ^= t; }
#pragma unroll
	for(int k = 0; k < 16; k += 2) { uint32_t t = ((m[k] >> 1) ^ m[k + 1]) & 0x5555u; m[k] ^= t << 1; m[k + 1] ^= t; }
	const size_t kBytes = (size_t)nInPad * 8;
#pragma unroll
	for(int j = 0; j < 16; j++)
		*reinterpret_cast<uint2*>(B + ((size_t)r * 16 + j) * kBytes + (size_t)i * 8) = t4_spread16(m[j]);
}

// ------------------------------------------------------------------ GEMM
__device__ __forceinline__ uint32_t t4_saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool t4_wait(uint32_t bar, uint32_t parity) {
	for(unsigned i = 0; i < T4_WAIT; i++) {
		uint32_t ok;
		asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
		             : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
		if(ok) return true;
	}
	atomicExch(&g_tc4_error, 1u);
	return false;
}

__device__ __forceinline__ void t4_arrive(uint32_t bar) {
	asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" :: "r"(bar) : "memory");
}

// K-major operand in shared memory, 128-byte swizzle: 8-row atoms 1024 bytes apart
__device__ __forceinline__ uint64_t t4_desc(uint32_t saddr) {
	uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
	d |= (uint64_t)1 << 16;
	d |= (uint64_t)(1024 >> 4) << 32;
	d |= (uint64_t)1 << 46;
	d |= (uint64_t)2 << 61;
	return d;
}

// instruction descriptor of the block-scaled kinds: A and B e2m1 (mxf4 code
// 1), K-major, N >> 3, ue8m0 scale factors, M >> 4, scale-factor ids 0
template<int BN> __device__ __forceinline__ uint32_t t4_idesc() {
	return (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) | (1u << 23) | ((uint32_t)(T4_BM >> 4) << 24);
}

// tile t -> (word tile mt, recovery tile nt): groups of groupM word tiles walk
// the recovery tiles together
__device__ __forceinline__ void t4_tile(unsigned t, unsigned mTiles, unsigned nTiles, unsigned groupM, unsigned& mt,
                                        unsigned& nt) {
	const unsigned grp = t / (groupM * nTiles);
	const unsigned gm = min(groupM, mTiles - grp * groupM);
	const unsigned within = t - grp * groupM * nTiles;
	mt = grp * groupM + within % gm;
	nt = within / gm;
}

// bounded wait that also gives up when another role of the CTA has given up
// (flag in shared memory), so that one failed wait ends the whole CTA quickly
__device__ __forceinline__ bool t4_wait_ab(uint32_t bar, uint32_t parity, volatile uint32_t* abortFlag) {
	for(unsigned i = 0; i < T4_WAIT; i++) {
		uint32_t ok;
		asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
		             : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
		if(ok) return true;
		if((i & 1023u) == 1023u && *abortFlag) return false;
	}
	atomicExch(&g_tc4_error, 1u);
	*abortFlag = 1u;
	return false;
}

// Persistent GEMM: one CTA per SM.  Warp 0 (one thread) takes tiles from a
// global counter (tile = atomicAdd(counter) - tileBase, so an SM that another
// kernel holds for a while simply takes fewer tiles), publishes each tile
// number in a ring of TR slots, and streams the tile's k-blocks through the
// stage ring without stopping at tile boundaries; warp 1 (one thread) reads
// the tile numbers and issues the MMAs of tile j into TMEM accumulator
// j % NACC, first waiting until the epilogue has read that accumulator's
// previous tile; warps 2-5 (each the TMEM lane quarter warp % 4) read the tile
// numbers and the accumulators out of TMEM.  With two accumulators the MMAs
// of the next tile run while the epilogue writes the previous one.  Each CTA's producer
// does exactly one counter fetch beyond its last tile (the one that ends
// it), so a launch advances the counter by tiles + CTAs.
template<int BN>
__global__ void __launch_bounds__(T4_THREADS, 1) k_tc4_gemm(const __grid_constant__ CUtensorMap tmA,
                                                          const __grid_constant__ CUtensorMap tmB,
                                                          uint16_t* __restrict__ rec, size_t recPitch, unsigned R,
                                                          unsigned kBlocks, unsigned mTiles, unsigned nTiles,
                                                          unsigned groupM, size_t w0, size_t nWords, int accumulate,
                                                          unsigned* __restrict__ tileCounter, unsigned tileBase)
{
	typedef T4Shape<BN> Sh;
	constexpr int NST = Sh::NST, STAGE = Sh::STAGE, NACC = Sh::NACC;
	extern __shared__ __align__(1024) uint8_t smem_raw[];
	const uint32_t raw = t4_saddr(smem_raw);
	const uint32_t pad = (1024u - (raw & 1023u)) & 1023u;
	uint8_t* sm = smem_raw + pad;
	const uint32_t sbase = raw + pad;
	const uint32_t barBase = sbase + NST * STAGE;
	auto bar = [&](int k) -> uint32_t { return barBase + 8u * (uint32_t)k; };
	volatile uint32_t* tileIds = reinterpret_cast<volatile uint32_t*>(sm + NST * STAGE + Sh::NBARS * 8);
	uint32_t* tslot = const_cast<uint32_t*>(tileIds) + T4_TR;
	volatile uint32_t* abortFlag = tslot + 1;
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const unsigned nAll = mTiles * nTiles;

	if(threadIdx.x == 0) {
		for(int k = 0; k < Sh::NBARS; k++) {
			unsigned count = 1;
			if(k == Sh::BAR_TEMPTY || k == Sh::BAR_TEMPTY + 1) count = 4;
			if(k >= Sh::BAR_IDEMPTY && k < Sh::BAR_IDEMPTY + T4_TR) count = 5;
			asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(bar(k)), "r"(count) : "memory");
		}
		*abortFlag = 0u;
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
		asm volatile("prefetch.tensormap [%0];" :: "l"(&tmA) : "memory");
		asm volatile("prefetch.tensormap [%0];" :: "l"(&tmB) : "memory");
	}
	if(warp == 1) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" :: "r"(t4_saddr(tslot)), "r"(512u) : "memory");
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
	}
	asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
	__syncthreads();
	asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
	const uint32_t tmem = *tslot;

	// scale factors: TMEM columns 448-511 of every lane hold ue8m0 1.0 bytes
	// (A's at column 448, B's at 480); each epilogue warp fills its own lane
	// quarter
	if(warp >= 2) {
		const uint32_t one = 0x7F7F7F7Fu;
		const uint32_t lane0 = (uint32_t)(32 * (warp & 3)) << 16;
#pragma unroll
		for(int q = 0; q < 2; q++)
			asm volatile("tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], "
			             "{%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1};"
			             :: "r"(tmem + lane0 + T4_SFA_COL + 32 * q), "r"(one) : "memory");
		asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
	}
	asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
	__syncthreads();
	asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

	if(warp == 0) {
		if(lane == 0) {
			// producer: tile numbers, then k-block g of the CTA's sequence into stage g % NST
			uint32_t g = 0;
			bool ok = true;
			for(uint32_t j = 0; ok; j++) {
				const unsigned slot = j % T4_TR;
				if(j >= T4_TR && !t4_wait_ab(bar(Sh::BAR_IDEMPTY + slot), ((j / T4_TR) - 1) & 1, abortFlag)) {
					ok = false;
					break;
				}
				const unsigned t = atomicAdd(tileCounter, 1u) - tileBase;
				const bool more = t < nAll;
				tileIds[slot] = more ? t : T4_NO_TILE;
				t4_arrive(bar(Sh::BAR_IDFULL + slot));
				if(!more) break;
				unsigned mt, nt;
				t4_tile(t, mTiles, nTiles, groupM, mt, nt);
				for(unsigned kb = 0; kb < kBlocks; kb++, g++) {
					const unsigned s = g % NST;
					if(g >= NST && !t4_wait_ab(bar(Sh::BAR_EMPTY + s), ((g / NST) - 1) & 1, abortFlag)) {
						ok = false;
						break;
					}
					const uint32_t full = bar(Sh::BAR_FULL + s);
					const uint32_t dA = sbase + s * STAGE, dB = dA + T4_STAGE_A;
					asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}"
					             :: "r"(full), "r"((uint32_t)STAGE) : "memory");
					const int x = (int)(kb * T4_KB);
					asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
					             :: "r"(dA), "l"(&tmA), "r"(x), "r"((int)(mt * T4_BM)), "r"(full) : "memory");
					asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
					             :: "r"(dB), "l"(&tmB), "r"(x), "r"((int)(nt * BN)), "r"(full) : "memory");
				}
			}
			if(!ok) {
				// let the copies still in flight land before the CTA ends
				for(uint32_t h = g > NST ? g - NST : 0; h < g; h++)
					t4_wait(bar(Sh::BAR_FULL + h % NST), (h / NST) & 1);
			}
		}
	} else if(warp == 1) {
		if(lane == 0) {
			// MMA issuer: tile j accumulates in TMEM columns (j % NACC) * 256 ..
			const uint32_t idesc = t4_idesc<BN>();
			const uint32_t sfa = tmem + T4_SFA_COL, sfb = tmem + T4_SFB_COL;
			uint32_t g = 0;
			bool ok = true;
			for(uint32_t j = 0; ok; j++) {
				const unsigned slot = j % T4_TR;
				if(!t4_wait_ab(bar(Sh::BAR_IDFULL + slot), (j / T4_TR) & 1, abortFlag)) { ok = false; break; }
				const unsigned t = tileIds[slot];
				t4_arrive(bar(Sh::BAR_IDEMPTY + slot));
				if(t == T4_NO_TILE) break;
				const unsigned buf = j % NACC, use = j / NACC;
				// the epilogue has read this accumulator's previous tile
				if(use >= 1 && !t4_wait_ab(bar(Sh::BAR_TEMPTY + buf), (use - 1) & 1, abortFlag)) { ok = false; break; }
				asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
				const uint32_t dacc = tmem + buf * T4_ACC_STRIDE;
				for(unsigned kb = 0; kb < kBlocks; kb++, g++) {
					const unsigned s = g % NST;
					if(!t4_wait_ab(bar(Sh::BAR_FULL + s), (g / NST) & 1, abortFlag)) { ok = false; break; }
					asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
					const uint32_t aS = sbase + s * STAGE, bS = aS + T4_STAGE_A;
#pragma unroll
					for(int k = 0; k < 4; k++) {
						const uint64_t ad = t4_desc(aS + k * 32), bd = t4_desc(bS + k * 32);
						const uint32_t acc = (kb | k) != 0;
						asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %6, 0;\n\t"
						             "tcgen05.mma.cta_group::1.kind::mxf4.block_scale.scale_vec::2X [%0], %1, %2, %3, [%4], [%5], p;\n\t}"
						             :: "r"(dacc), "l"(ad), "l"(bd), "r"(idesc), "r"(sfa), "r"(sfb), "r"(acc) : "memory");
					}
					asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
					             :: "r"(bar(Sh::BAR_EMPTY + s)) : "memory");
				}
				if(ok)
					asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
					             :: "r"(bar(Sh::BAR_TFULL + buf)) : "memory");
			}
			// every MMA this thread issued has completed before TMEM is freed
			asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
			             :: "r"(bar(Sh::BAR_DRAIN)) : "memory");
			t4_wait(bar(Sh::BAR_DRAIN), 0);
		}
	} else {
		// epilogue: thread (warp, lane) owns word mt*128 + 32*(warp%4) + lane
		// and the BN accumulator columns of its TMEM lane = BN / 16 recovery words
		const unsigned quarter = warp & 3;
		const uint32_t lane0 = (uint32_t)(32 * quarter) << 16;
		for(uint32_t j = 0;; j++) {
			const unsigned slot = j % T4_TR;
			if(!__all_sync(0xffffffffu, t4_wait_ab(bar(Sh::BAR_IDFULL + slot), (j / T4_TR) & 1, abortFlag))) break;
			const unsigned t = tileIds[slot];
			__syncwarp();
			if(lane == 0) t4_arrive(bar(Sh::BAR_IDEMPTY + slot));
			if(t == T4_NO_TILE) break;
			unsigned mt, nt;
			t4_tile(t, mTiles, nTiles, groupM, mt, nt);
			const unsigned buf = j % NACC, use = j / NACC;
			if(!__all_sync(0xffffffffu, t4_wait_ab(bar(Sh::BAR_TFULL + buf), use & 1, abortFlag))) break;
			asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
			const size_t w = w0 + (size_t)mt * T4_BM + 32 * quarter + lane;
#pragma unroll 1
			for(int q = 0; q < BN / 32; q++) {
				uint32_t v[32];
				asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 "
				             "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
				             "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
				             : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
				               "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
				               "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
				               "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
				             : "r"(tmem + lane0 + buf * T4_ACC_STRIDE + 32 * q));
				asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
				// parity of an exact integer n < 2^23 held in fp32: n + 2^23 has
				// unit ulp, so bit 0 of its encoding is bit 0 of n (one full-rate
				// add instead of a float-to-integer conversion per column)
				uint32_t word0 = 0, word1 = 0;
#pragma unroll
				for(int c = 0; c < 16; c++) {
					word0 |= (__float_as_uint(__fadd_rn(__uint_as_float(v[c]), 8388608.0f)) & 1u) << c;
					word1 |= (__float_as_uint(__fadd_rn(__uint_as_float(v[16 + c]), 8388608.0f)) & 1u) << c;
				}
				const unsigned r0 = nt * Sh::RPT + 2 * q;
				if(w < nWords) {
					if(r0 < R) {
						uint16_t* p = rec + (size_t)r0 * recPitch + w;
						*p = accumulate ? (uint16_t)(*p ^ word0) : (uint16_t)word0;
					}
					if(r0 + 1 < R) {
						uint16_t* p = rec + (size_t)(r0 + 1) * recPitch + w;
						*p = accumulate ? (uint16_t)(*p ^ word1) : (uint16_t)word1;
					}
				}
			}
			// this warp's TMEM reads are done: the accumulator may take a new tile
			asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
			__syncwarp();
			if(lane == 0) t4_arrive(bar(Sh::BAR_TEMPTY + buf));
		}
	}
	__syncwarp();
	asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
	__syncthreads();
	asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
	if(warp == 1)
		asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(512u) : "memory");
}

// ------------------------------------------------------------------ host
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn t4_encoder() {
	static EncodeTiledFn fn = nullptr;
	if(!fn) {
		void* p = nullptr;
		cudaDriverEntryPointQueryResult q;
		if(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
		   q == cudaDriverEntryPointSuccess)
			fn = reinterpret_cast<EncodeTiledFn>(p);
	}
	return fn;
}

static int t4_map(CUtensorMap* m, const void* base, size_t rowBytes, size_t rows, unsigned boxRows) {
	EncodeTiledFn enc = t4_encoder();
	if(!enc) { set_error("tensor method: cuTensorMapEncodeTiled is not available"); return -1; }
	const cuuint64_t dims[2] = {rowBytes, rows};
	const cuuint64_t strides[1] = {rowBytes};
	const cuuint32_t box[2] = {T4_KB, boxRows};
	const cuuint32_t estr[2] = {1, 1};
	CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, const_cast<void*>(base), dims, strides, box, estr,
	                 CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
	                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
	if(r != CUDA_SUCCESS) { set_error("tensor method: cuTensorMapEncodeTiled failed (%d)", (int)r); return -1; }
	return 0;
}

// scratch: [tile counter, 1 KiB] [B: 16 x roundup(R, 48) rows of kBytes] [A chunk]
#define T4_HDR_BYTES 1024
static size_t t4_kbytes(unsigned nIn) { return (size_t)round_up(nIn ? nIn : 1, 16) * 8; }
static unsigned t4_rpad(unsigned R) { return (unsigned)round_up(R ? R : 1, T4_RCOMMON); }

static std::atomic<int> g_tc4_shape{0};
int set_tc4_shape(int shape) { return g_tc4_shape.exchange(shape); }
static std::atomic<int> g_tc4_group{0};
int set_tc4_group(int groupM) { return g_tc4_group.exchange(groupM); }

// Tile shape for kBlocks k-blocks (16 inputs each) per tile.  The 192-row
// tile with two accumulators hides each tile's read-out behind the next
// tile's MMAs, but its A tiles are loaded 4/3 as often per MMA and its MMAs
// are narrower; measured on GB300 it is slower on every shape tried (4096 x
// 4096 x 256 KiB: 187.6 against 146.5 ms; 512 x 192 x 512 KiB: 2.72 against
// 2.32 ms; 2000 x 200 x 2 MiB: 42.6 against 35.6 ms; 1000 x 100 x 1 MiB:
// 6.51 against 5.67 ms), so the automatic choice is the 256-row tile.
int tc4_shape_for(unsigned kBlocks) {
	(void)kBlocks;
	const int s = g_tc4_shape.load();
	return s == 2 ? 2 : 1;
}
static size_t t4_bbytes(unsigned R, unsigned nIn) {
	return round_up((size_t)t4_rpad(R) * 16 * t4_kbytes(nIn), 1024);
}

size_t tc4_scratch_bytes(unsigned R, unsigned nIn, size_t nWords) {
	const size_t aFull = round_up(nWords ? nWords : 1, T4_BM) * t4_kbytes(nIn);
	const size_t aMax = std::max<size_t>(T4_A_CHUNK_BYTES, (size_t)T4_BM * t4_kbytes(nIn));
	return T4_HDR_BYTES + t4_bbytes(R, nIn) + round_up(std::min(aFull, aMax), 1024);
}

size_t tc4_scratch_chunked_bytes(unsigned R, unsigned nIn, size_t nWords, size_t aChunkBytes) {
	const size_t aMin = std::max<size_t>(aChunkBytes, (size_t)T4_BM * t4_kbytes(nIn));
	return std::min(tc4_scratch_bytes(R, nIn, nWords), T4_HDR_BYTES + t4_bbytes(R, nIn) + round_up(aMin, 1024));
}

unsigned tc4_launches(unsigned R, unsigned nIn, size_t nWords, size_t scratchBytes) {
	if(!R || !nWords || !nIn) return 0;
	const size_t kBytes = t4_kbytes(nIn), bBytes = t4_bbytes(R, nIn);
	if(scratchBytes < T4_HDR_BYTES + bBytes + (size_t)T4_BM * kBytes) return 0;
	size_t wChunk = (scratchBytes - T4_HDR_BYTES - bBytes) / kBytes / T4_BM * T4_BM;
	wChunk = std::min(wChunk, round_up(nWords, T4_BM));
	return 1 + 2 * (unsigned)((nWords + wChunk - 1) / wChunk);   // coefficients, then per chunk: inputs + GEMM
}

int tc4_muladd(const uint16_t* in, size_t inPitch, unsigned nIn, const uint16_t* coeff, uint16_t* rec, size_t recPitch,
               unsigned R, size_t nWords, int accumulate, void* scratch, size_t scratchBytes, cudaStream_t st)
{
	if(!R || !nWords) return 0;
	if(!nIn) {
		if(!accumulate) P2C_CUDA_TRY(cudaMemset2DAsync(rec, recPitch * 2, 0, nWords * 2, R, st));
		return 0;
	}
	if(nIn >= (1u << 19)) {
		// a column sums up to 16 x nIn ones; the epilogue's parity read needs
		// the sum below 2^23
		set_error("tensor method (mxf4): %u inputs in one call, at most %u", nIn, (1u << 19) - 1);
		return -1;
	}
	const size_t kBytes = t4_kbytes(nIn);
	const unsigned nInPad = (unsigned)(kBytes / 8), rPad = t4_rpad(R);
	const size_t bBytes = t4_bbytes(R, nIn);
	const size_t minBytes = T4_HDR_BYTES + bBytes + (size_t)T4_BM * kBytes;
	if(!scratch || scratchBytes < minBytes) {
		set_error("tensor method (mxf4) needs at least %zu bytes of scratch, %zu given", minBytes, scratchBytes);
		return -1;
	}
	unsigned* counter = reinterpret_cast<unsigned*>(scratch);
	uint8_t* B = reinterpret_cast<uint8_t*>(scratch) + T4_HDR_BYTES;
	uint8_t* A = B + bBytes;
	// words per chunk: what the rest of the scratch holds, in whole 128-word tiles
	size_t wChunk = (scratchBytes - T4_HDR_BYTES - bBytes) / kBytes / T4_BM * T4_BM;
	wChunk = std::min(wChunk, round_up(nWords, T4_BM));
	const size_t nB = (size_t)rPad * nInPad;
	k_tc4_prep_coeff<<<(unsigned)((nB + 255) / 256), 256, 0, st>>>(coeff, R, nIn, rPad, nInPad, B);
	P2C_CUDA_TRY(cudaGetLastError());
	const unsigned kBlocks = (unsigned)(kBytes / T4_KB);
	const int shape = tc4_shape_for(kBlocks);
	const unsigned bn = shape == 1 ? 256 : 192, rpt = bn / 16;
	const size_t smem = shape == 1 ? T4Shape<256>::SMEM : T4Shape<192>::SMEM;
	if(shape == 1) P2C_CUDA_TRY(cudaFuncSetAttribute(k_tc4_gemm<256>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
	else P2C_CUDA_TRY(cudaFuncSetAttribute(k_tc4_gemm<192>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
	CUtensorMap tmB;
	if(t4_map(&tmB, B, kBytes, (size_t)rPad * 16, bn)) return -1;
	int dev = 0, nSM = 0;
	P2C_CUDA_TRY(cudaGetDevice(&dev));
	P2C_CUDA_TRY(cudaDeviceGetAttribute(&nSM, cudaDevAttrMultiProcessorCount, dev));
	// recovery tiles: B has rows for rPad >= nTiles * rpt slices
	const unsigned nTiles = (R + rpt - 1) / rpt;
	// word tiles per raster group: their A tiles (128 x kBytes each) stay in
	// L2 (about 48 MiB of it) while the group walks the recovery tiles, so A
	// is read from HBM once and each B tile once per group
	unsigned groupM = (unsigned)std::min<size_t>(64, std::max<size_t>(8, (48ull << 20) / ((size_t)T4_BM * kBytes)));
	if(g_tc4_group.load() > 0) groupM = (unsigned)g_tc4_group.load();
	// the tile counter starts at 0 for this call; each launch advances it by
	// its tiles + CTAs (every CTA's last fetch finds no tile)
	P2C_CUDA_TRY(cudaMemsetAsync(counter, 0, sizeof(unsigned), st));
	unsigned base = 0;
	for(size_t w0 = 0; w0 < nWords; w0 += wChunk) {
		const size_t rows = std::min(wChunk, round_up(nWords - w0, T4_BM));
		if((reinterpret_cast<uintptr_t>(in) & 15) == 0 && (inPitch & 7) == 0) {
			dim3 pg((unsigned)(rows / 128), (nInPad + 63) / 64);
			k_tc4_prep_in_v<<<pg, 256, 0, st>>>(in, inPitch, nIn, nWords, w0, A, kBytes);
		} else {
			dim3 pg((unsigned)(rows / 64), (nInPad + 63) / 64);
			k_tc4_prep_in<<<pg, 256, 0, st>>>(in, inPitch, nIn, nWords, w0, A, kBytes);
		}
		P2C_CUDA_TRY(cudaGetLastError());
		CUtensorMap tmA;
		if(t4_map(&tmA, A, kBytes, rows, T4_BM)) return -1;
		const unsigned mTiles = (unsigned)(rows / T4_BM);
		const unsigned nAll = mTiles * nTiles;
		// one CTA per SM (its shared memory allows no second)
		const unsigned grid = (unsigned)std::min<size_t>((size_t)nAll, (size_t)std::max(nSM, 1));
		if(shape == 1)
			k_tc4_gemm<256><<<grid, T4_THREADS, smem, st>>>(tmA, tmB, rec, recPitch, R, kBlocks, mTiles, nTiles, groupM, w0,
			                                                nWords, accumulate, counter, base);
		else
			k_tc4_gemm<192><<<grid, T4_THREADS, smem, st>>>(tmA, tmB, rec, recPitch, R, kBlocks, mTiles, nTiles, groupM, w0,
			                                                nWords, accumulate, counter, base);
		P2C_CUDA_TRY(cudaGetLastError());
		base += nAll + grid;
	}
	return 0;
}

// ------------------------------------------------------------------ peak
// Calibration of the roofline denominator: one CTA per SM issues `iters`
// MMAs of the default tile shape (M=128, N=256, K=64, kind::mxf4, unit scales) on
// operands resident in shared memory, back to back into one accumulator, and
// waits (bounded) for their completion.  No global memory traffic: the rate
// is the tensor pipe's for this instruction.
__global__ void __launch_bounds__(128, 1) k_tc4_mma_rate(unsigned iters)
{
	extern __shared__ __align__(1024) uint8_t smem_raw[];
	const uint32_t raw = t4_saddr(smem_raw);
	const uint32_t pad = (1024u - (raw & 1023u)) & 1023u;
	uint8_t* sm = smem_raw + pad;
	const uint32_t sbase = raw + pad;
	constexpr int STAGE = T4Shape<256>::STAGE;
	const uint32_t doneBar = sbase + STAGE;
	uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + STAGE + 8);
	const int warp = threadIdx.x >> 5;
	for(int e = threadIdx.x; e < STAGE / 16; e += 128) reinterpret_cast<uint4*>(sm)[e] = make_uint4(0, 0, 0, 0);
	if(threadIdx.x == 0) {
		asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(doneBar) : "memory");
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	}
	asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
	if(warp == 0) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" :: "r"(t4_saddr(tslot)), "r"(512u) : "memory");
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
	}
	asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
	__syncthreads();
	asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
	const uint32_t tmem = *tslot;
	{
		const uint32_t one = 0x7F7F7F7Fu;
		const uint32_t lane0 = (uint32_t)(32 * warp) << 16;
#pragma unroll
		for(int q = 0; q < 2; q++)
			asm volatile("tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], "
			             "{%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1};"
			             :: "r"(tmem + lane0 + T4_SFA_COL + 32 * q), "r"(one) : "memory");
		asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
	}
	asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
	__syncthreads();
	asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
	if(threadIdx.x == 0) {
		const uint32_t idesc = t4_idesc<256>();
		const uint64_t ad = t4_desc(sbase), bd = t4_desc(sbase + T4_STAGE_A);
		for(unsigned it = 0; it < iters; it++) {
			const uint32_t acc = it != 0;
			asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %6, 0;\n\t"
			             "tcgen05.mma.cta_group::1.kind::mxf4.block_scale.scale_vec::2X [%0], %1, %2, %3, [%4], [%5], p;\n\t}"
			             :: "r"(tmem), "l"(ad), "l"(bd), "r"(idesc), "r"(tmem + T4_SFA_COL), "r"(tmem + T4_SFB_COL), "r"(acc) : "memory");
		}
		asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" :: "r"(doneBar) : "memory");
	}
	__syncwarp();
	t4_wait(doneBar, 0);
	asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
	__syncthreads();
	if(warp == 0)
		asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(512u) : "memory");
}

int tc4_mma_rate(double* macsPerSec, cudaStream_t st) {
	int dev = 0, sms = 0;
	P2C_CUDA_TRY(cudaGetDevice(&dev));
	P2C_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
	const size_t smem = T4Shape<256>::STAGE + 8 + 16 + 1024;
	P2C_CUDA_TRY(cudaFuncSetAttribute(k_tc4_mma_rate, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
	const unsigned iters = 20000;
	cudaEvent_t e0, e1;
	P2C_CUDA_TRY(cudaEventCreate(&e0));
	P2C_CUDA_TRY(cudaEventCreate(&e1));
	float best = 0.f;
	for(int rep = 0; rep < 3; rep++) {
		cudaEventRecord(e0, st);
		k_tc4_mma_rate<<<sms, 128, smem, st>>>(iters);
		cudaEventRecord(e1, st);
		cudaEventSynchronize(e1);
		float ms = 0.f;
		cudaEventElapsedTime(&ms, e0, e1);
		if(rep == 0 || ms < best) best = ms;
	}
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	P2C_CUDA_TRY(cudaGetLastError());
	*macsPerSec = best > 0.f ? (double)iters * sms * T4_BM * 256 * 64 / (best * 1e-3) : 0.0;
	return 0;
}

int tc4_error_take() {
	unsigned v = 0, z = 0;
	if(cudaMemcpyFromSymbol(&v, g_tc4_error, sizeof(v)) != cudaSuccess) return -1;
	if(v) cudaMemcpyToSymbol(g_tc4_error, &z, sizeof(z));
	return (int)v;
}

} // namespace p2c
