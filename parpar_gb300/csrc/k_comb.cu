// GF(2^16) multiply-accumulate of a batch of input rows into recovery rows:
//     rec[r][w] (^)= sum_i c(r,i) * in[i][w]
// (the hot loop of gf16/controller_cpu.cpp:488-515 / the OpenCL mul-group
// kernel gf16/controller_ocl_init.cpp:588-671), as an XOR-combination-table
// ("comb") kernel.
//
// Algebra.  Multiplication by c is linear over GF(2): with c = sum_k c_k x^k,
//     sum_i c(r,i) in_i = sum_k x^k P[r][k],   P[r][k] = XOR_{i : bit k of c(r,i)} in_i
// so the bulk of the work is 16 binary (XOR-only) combinations per recovery
// row, followed by a 15-step Horner (multiply by x, XOR) per word at the end.
// Inputs are taken 8 at a time: a CTA builds, in shared memory, the 256
// possible XOR combinations T[m] = XOR_{t : bit t of m} in_{8g+t} of its word
// tile, and each (recovery row, k) pair then costs one table row read:
//     P[r][k] ^= T[ idx[r][g][k] ],  idx[r][g][k] = sum_t bit_k(c(r,8g+t)) << t
// (the index bytes are prepared per launch by k_make_idx / k_coeff_to_idx).
//
// Roofline.  Per word mul-add the kernel reads 16/8 table entries of 2 bytes
// from shared memory = 4 bytes, against the SM's 128 B/clk shared-memory
// port: <= 32 word mul-adds / clk / SM.  HBM traffic per launch is
// (nIn + 2R) rows; global index traffic is 2 bytes per (r, i) per word tile.
//
// Layout: CTA tile = 64 words (32 lanes x one u32 = 2 words) x RT recovery
// rows (NW warps x RPW rows per warp); P accumulators live in registers
// (16 u32 per row per lane).  Two table buffers interleave inside each
// 256-byte table row (bytes 0-127 buffer 0, 128-255 buffer 1), so one PRMT
// forms the full shared-memory address (m << 8 | buffer << 7 | lane << 2).
#include "common.cuh"
#include "kernels.h"

#include <atomic>

namespace p2c {

// One work unit: word tile `tile` (64 words) x recovery rows [rbase, rbase+RT)
// of one job, all of its inputs.  Ends with every thread past a barrier and no
// shared memory in use, so a CTA may run units back to back.
template<int RPW, int NW>
__device__ __forceinline__ void comb_unit(
	const uint16_t* __restrict__ in, size_t inPitch, unsigned nIn,
	const uint4* __restrict__ idx, unsigned G,
	uint16_t* __restrict__ rec, size_t recPitch, unsigned R, int accumulate,
	size_t tile, unsigned rbase, uint8_t* smem)
{
	constexpr int RT = RPW * NW;              // recovery rows per CTA
	uint8_t* tbl = smem;                                    // 256 rows x 256 B
	uint4* idxs = reinterpret_cast<uint4*>(smem + 65536);   // [2][RT]

	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const size_t colWord = tile * P2C_TILE_WORDS + lane * 2;  // this lane's 2 words
	const uint32_t* in32 = reinterpret_cast<const uint32_t*>(in);

	uint32_t acc[RPW][16];
#pragma unroll
	for(int s = 0; s < RPW; s++)
#pragma unroll
		for(int k = 0; k < 16; k++) acc[s][k] = 0;

	constexpr int NB = NW >= 8 ? 8 : (NW >= 4 ? 4 : (NW >= 2 ? 2 : 1)); // build warps
	constexpr int HPW = 16 / NB;             // high-nibble values built per build warp
	// the 8 input words of group g for this lane (zero past nIn)
	auto load_group = [&](unsigned g, uint32_t (&x)[8]) {
#pragma unroll
		for(int t = 0; t < 8; t++) {
			unsigned i = g * 8 + t;
			x[t] = i < nIn ? __ldg(in32 + ((size_t)i * inPitch + colWord) / 2) : 0u;
		}
	};
	// build table buffer `b` from x (build warps only): rows (h << 4 | n) for
	// this warp's HPW high nibbles h, the 16 low nibbles n in Gray-code order so
	// that each row costs one XOR
	auto build = [&](int b, const uint32_t (&x)[8]) {
		uint8_t* base = tbl + b * 128 + lane * 4;
#pragma unroll
		for(int hh = 0; hh < HPW; hh++) {
			const int h = warp * HPW + hh;
			uint32_t hv = 0;
#pragma unroll
			for(int t = 0; t < 4; t++) if(h >> t & 1) hv ^= x[4 + t];
			uint32_t lv = hv;
			uint8_t* rowp = base + h * 16 * 256;
			*reinterpret_cast<uint32_t*>(rowp) = lv;       // n = 0
#pragma unroll
			for(int n = 1; n < 16; n++) {
				const int gray = n ^ (n >> 1);
				const int bit = (n & 1) ? 0 : (n & 2) ? 1 : (n & 4) ? 2 : 3;
				lv ^= x[bit];
				*reinterpret_cast<uint32_t*>(rowp + gray * 256) = lv;
			}
		}
	};
	auto stage_idx = [&](unsigned g, int b) {
		for(int j = threadIdx.x; j < RT; j += NW * 32) {
			unsigned r = rbase + j;
			idxs[b * RT + j] = r < R ? __ldg(idx + (size_t)r * G + g) : make_uint4(0, 0, 0, 0);
		}
	};

	uint32_t x[8];
	if(warp < NB) { load_group(0, x); build(0, x); }
	stage_idx(0, 0);
	__syncthreads();

	const uint32_t lw0 = (uint32_t)lane * 4, lw1 = lw0 + 128;
	for(unsigned g = 0; g < G; g++) {
		const int b = g & 1;
		const bool more = g + 1 < G;
		if(more && warp < NB) load_group(g + 1, x);
		const uint32_t lw = b ? lw1 : lw0;
		// lookups for group g
#pragma unroll
		for(int s = 0; s < RPW; s++) {
			const int j = warp * RPW + s;
			if(rbase + j < R) {
				const uint4 q = idxs[b * RT + j];
				const uint32_t qq[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
				for(int k = 0; k < 16; k++) {
					// selector: byte0 <- lw.byte0, byte1 <- q.byte(k&3), bytes 2,3 <- lw.byte1 (=0)
					const uint32_t sel = 4u | ((uint32_t)(k & 3) << 4) | (5u << 8) | (5u << 12);
					const uint32_t addr = __byte_perm(qq[k >> 2], lw, sel);
					acc[s][k] ^= *reinterpret_cast<const uint32_t*>(tbl + addr);
				}
			}
		}
		if(more) {
			if(warp < NB) build(b ^ 1, x);
			stage_idx(g + 1, b ^ 1);
		}
		__syncthreads();
	}

	// epilogue: rec[r] (^)= sum_k x^k P[r][k]
	uint32_t* rec32 = reinterpret_cast<uint32_t*>(rec);
#pragma unroll
	for(int s = 0; s < RPW; s++) {
		const unsigned r = rbase + warp * RPW + s;
		if(r < R) {
			uint32_t v = acc[s][15];
#pragma unroll
			for(int k = 14; k >= 0; k--) v = mul2x2(v) ^ acc[s][k];
			uint32_t* p = rec32 + ((size_t)r * recPitch + colWord) / 2;
			if(accumulate) v ^= *p;
			*p = v;
		}
	}
}

template<int RPW, int NW>
__global__ void __launch_bounds__(NW * 32, 1) k_comb_muladd(
	const uint16_t* __restrict__ in, size_t inPitch, unsigned nIn,
	const uint4* __restrict__ idx, unsigned G,
	uint16_t* __restrict__ rec, size_t recPitch, unsigned R, int accumulate)
{
	extern __shared__ __align__(16) uint8_t smem[];
	comb_unit<RPW, NW>(in, inPitch, nIn, idx, G, rec, recPitch, R, accumulate, blockIdx.x, blockIdx.y * (RPW * NW), smem);
}

// Persistent batched form: a grid of one CTA per SM (x occupancy) takes work
// units (job, word tile, recovery block) from a device counter until the
// list is exhausted.  Jobs are laid out job-major, largest first, so the
// largest units are handed out first and the tail is made of small ones.
// The counter is an atomicAdd ticket; there is no waiting on other CTAs.
template<int RPW, int NW>
__global__ void __launch_bounds__(NW * 32, 1) k_comb_batched(
	const BatchJob* __restrict__ jobs, unsigned nJobs, unsigned long long totalUnits,
	unsigned long long* __restrict__ counter)
{
	constexpr int RT = RPW * NW;
	extern __shared__ __align__(16) uint8_t smem[];
	__shared__ unsigned long long s_unit;
	__shared__ unsigned s_job;
	for(;;) {
		if(threadIdx.x == 0) {
			unsigned long long u = atomicAdd(counter, 1ull);
			s_unit = u;
			// last job whose first unit <= u (unitBase ascending)
			unsigned lo = 0, hi = nJobs;
			while(hi - lo > 1) {
				unsigned mid = (lo + hi) >> 1;
				if(jobs[mid].unitBase <= u) lo = mid; else hi = mid;
			}
			s_job = lo;
		}
		__syncthreads();
		const unsigned long long u = s_unit;
		if(u >= totalUnits) break;
		const BatchJob& J = jobs[s_job];
		const unsigned long long local = u - J.unitBase;
		const unsigned rblocks = (J.R + RT - 1) / RT;
		const size_t tile = (size_t)(local / rblocks);
		const unsigned rb = (unsigned)(local % rblocks);
		comb_unit<RPW, NW>(J.in, J.inPitch, J.nIn, J.idx, (J.nIn + 7) / 8, J.rec, J.recPitch, J.R, J.accumulate,
		                   tile, rb * RT, smem);
		__syncthreads(); // s_unit / s_job are rewritten next round
	}
}

template<int RPW, int NW>
static int launch_comb(const uint16_t* in, size_t inPitch, unsigned nIn, const uint4* idx, uint16_t* rec,
                       size_t recPitch, unsigned R, size_t nWords, int accumulate, cudaStream_t st)
{
	constexpr int RT = RPW * NW;
	const size_t smem = 65536 + 2 * RT * sizeof(uint4);
	P2C_CUDA_TRY(cudaFuncSetAttribute(k_comb_muladd<RPW, NW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
	const unsigned G = (nIn + 7) / 8;
	dim3 grid((unsigned)((nWords + P2C_TILE_WORDS - 1) / P2C_TILE_WORDS), (R + RT - 1) / RT);
	k_comb_muladd<RPW, NW><<<grid, NW * 32, smem, st>>>(in, inPitch, nIn, idx, G, rec, recPitch, R, accumulate);
	P2C_CUDA_TRY(cudaGetLastError());
	return 0;
}


// ---------------------------------------------------------------------------
// Warp-specialised form: 4 builder warps produce the XOR tables (and stage the
// index bytes) into a two-buffer ring; NL lookup warps consume them.  Each
// buffer has a "full" mbarrier (128 builder arrivals) and an "empty" mbarrier
// (one arrival per lookup warp), so lookup warps never wait for one another,
// only for a table that is not built yet.  Every wait is bounded: after
// P2C_WAIT_LIMIT polls the kernel records an error in g_comb_error and the
// thread leaves (the host reports it; nothing spins forever).
#define P2C_WAIT_LIMIT (1u << 22)
__device__ unsigned g_comb_error;

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
	asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" :: "r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, unsigned limit = P2C_WAIT_LIMIT) {
	const unsigned a = smem_addr(bar);
	for(unsigned i = 0; i < limit; i++) {
		unsigned ok;
		asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
		             : "=r"(ok) : "r"(a), "r"(parity) : "memory");
		if(ok) return true;
	}
	atomicExch(&g_comb_error, 1u);
	return false;
}

// Self-test of the bounded wait: one warp waits on an mbarrier that nothing
// arrives on, with the same helper as the kernels above and `polls` as its
// limit; the wait gives up, records the error flag and the kernel returns.
__device__ unsigned g_wait_selftest;
__global__ void k_wait_selftest(unsigned polls) {
	__shared__ __align__(8) uint64_t bar;
	if(threadIdx.x == 0) mbar_init(&bar, 1);
	__syncthreads();
	const bool ok = mbar_wait(&bar, 0, polls);
	if(threadIdx.x == 0) g_wait_selftest = ok ? 1u : 2u;
}

int wait_selftest(unsigned polls, int* gaveUp, double* seconds) {
	cudaStream_t st;
	P2C_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
	cudaEvent_t e0, e1;
	cudaEventCreate(&e0);
	cudaEventCreate(&e1);
	const unsigned zero = 0;
	cudaMemcpyToSymbolAsync(g_wait_selftest, &zero, sizeof(zero), 0, cudaMemcpyHostToDevice, st);
	cudaEventRecord(e0, st);
	k_wait_selftest<<<1, 32, 0, st>>>(polls);
	cudaError_t le = cudaGetLastError();
	cudaEventRecord(e1, st);
	cudaError_t se = cudaStreamSynchronize(st);
	float ms = 0.f;
	cudaEventElapsedTime(&ms, e0, e1);
	unsigned out = 0;
	cudaMemcpyFromSymbol(&out, g_wait_selftest, sizeof(out));
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	cudaStreamDestroy(st);
	if(le != cudaSuccess || se != cudaSuccess) {
		set_error("wait self-test: %s", cudaGetErrorString(le != cudaSuccess ? le : se));
		return -1;
	}
	if(gaveUp) *gaveUp = out == 2 ? 1 : 0;
	if(seconds) *seconds = ms * 1e-3;
	return 0;
}

// WIDE = 1: each lane owns 4 words (LDS.64 per lookup, 128-word tiles,
// 512-byte table rows holding both buffers); WIDE = 0: 2 words (LDS.32,
// 64-word tiles, 256-byte rows).  ASMLD issues the table reads as explicit
// ld.shared with a 32-bit shared-window address.
template<int RPW, int NL, int WIDE, bool ASMLD>
__global__ void __launch_bounds__((NL + 4) * 32, 1) k_comb_ws(
	const uint16_t* __restrict__ in, size_t inPitch, unsigned nIn,
	const uint4* __restrict__ idx, unsigned G,
	uint16_t* __restrict__ rec, size_t recPitch, unsigned R, int accumulate, size_t limitWords)
{
	constexpr int RT = RPW * NL;
	constexpr int V = WIDE ? 2 : 1;                 // u32 per lane
	constexpr int TW = P2C_TILE_WORDS * V;          // words per tile
	constexpr int ROWB = 256 * V;                   // table row stride (both buffers)
	constexpr int TBL = 256 * ROWB;
	extern __shared__ __align__(16) uint8_t smem[];
	uint8_t* tbl = smem;
	uint4* idxs = reinterpret_cast<uint4*>(smem + TBL);           // [2][RT]
	uint64_t* bars = reinterpret_cast<uint64_t*>(smem + TBL + 2 * RT * sizeof(uint4)); // full[2], empty[2]
	const unsigned sbase = smem_addr(smem);

	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const size_t tile = blockIdx.x;
	const unsigned rbase = blockIdx.y * RT;
	const size_t colWord = tile * TW + lane * 2 * V;
	// rows are only guaranteed up to roundup(nWords, 64) words: with 128-word
	// tiles the upper half of the last tile may lie beyond the row
	const bool laneIn = colWord + 2 * V <= limitWords;

	if(threadIdx.x == 0) {
		mbar_init(&bars[0], 128);
		mbar_init(&bars[1], 128);
		mbar_init(&bars[2], NL);
		mbar_init(&bars[3], NL);
	}
	__syncthreads();

	if(warp >= NL) {
		// ---------------- builders: 4 warps, 4 high nibbles each
		const int bw = warp - NL;
		const int bt = threadIdx.x - NL * 32; // 0..127
		for(unsigned g = 0; g < G; g++) {
			const int b = g & 1;
			if(g >= 2 && !mbar_wait(&bars[2 + b], ((g >> 1) - 1) & 1)) return;
			uint32_t x[8][V];
#pragma unroll
			for(int t = 0; t < 8; t++) {
				unsigned i = g * 8 + t;
				if(WIDE) {
					uint2 v = (i < nIn && laneIn) ? __ldg(reinterpret_cast<const uint2*>(in + (size_t)i * inPitch + colWord)) : make_uint2(0, 0);
					x[t][0] = v.x; x[t][V - 1] = v.y;
				} else {
					x[t][0] = i < nIn ? __ldg(reinterpret_cast<const uint32_t*>(in + (size_t)i * inPitch + colWord)) : 0u;
				}
			}
			uint8_t* base = tbl + b * (ROWB / 2) + lane * 4 * V;
#pragma unroll
			for(int hh = 0; hh < 4; hh++) {
				const int h = bw * 4 + hh;
				uint32_t v[V];
#pragma unroll
				for(int c = 0; c < V; c++) {
					v[c] = 0;
#pragma unroll
					for(int t = 0; t < 4; t++) if(h >> t & 1) v[c] ^= x[4 + t][c];
				}
				uint8_t* rowp = base + h * 16 * ROWB;
				if(WIDE) *reinterpret_cast<uint2*>(rowp) = make_uint2(v[0], v[V - 1]);
				else *reinterpret_cast<uint32_t*>(rowp) = v[0];
#pragma unroll
				for(int n = 1; n < 16; n++) {
					const int gray = n ^ (n >> 1);
					const int bit = (n & 1) ? 0 : (n & 2) ? 1 : (n & 4) ? 2 : 3;
#pragma unroll
					for(int c = 0; c < V; c++) v[c] ^= x[bit][c];
					if(WIDE) *reinterpret_cast<uint2*>(rowp + gray * ROWB) = make_uint2(v[0], v[V - 1]);
					else *reinterpret_cast<uint32_t*>(rowp + gray * ROWB) = v[0];
				}
			}
			for(int j = bt; j < RT; j += 128) {
				unsigned r = rbase + j;
				idxs[b * RT + j] = r < R ? __ldg(idx + (size_t)r * G + g) : make_uint4(0, 0, 0, 0);
			}
			mbar_arrive(&bars[b]);  // release: this thread's table rows and index bytes
		}
		return;
	}

	// ---------------- lookups
	uint32_t acc[RPW][16][V];
#pragma unroll
	for(int s = 0; s < RPW; s++)
#pragma unroll
		for(int k = 0; k < 16; k++)
#pragma unroll
			for(int c = 0; c < V; c++) acc[s][k][c] = 0;
	const uint32_t lwb = (uint32_t)lane * 4 * V;

	auto lookups = [&](int b) {
		const uint32_t lw = lwb + b * (ROWB / 2);
#pragma unroll
		for(int s = 0; s < RPW; s++) {
			const int j = warp * RPW + s;
			if(rbase + j < R) {
				const uint4 q = idxs[b * RT + j];
				const uint32_t qq[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
				for(int k = 0; k < 16; k++) {
					uint32_t addr;
					if(WIDE) {
						// (m << 9) | lw: byte1 <- m << 1 is not a byte move, so build m << 8 and double it
						const uint32_t sel = 4u | ((uint32_t)(k & 3) << 4) | (5u << 8) | (5u << 12);
						addr = (__byte_perm(qq[k >> 2], 0, sel & 0xFFF0u | 5u) << 1) | lw;
					} else {
						const uint32_t sel = 4u | ((uint32_t)(k & 3) << 4) | (5u << 8) | (5u << 12);
						addr = __byte_perm(qq[k >> 2], lw, sel);
					}
					if(WIDE) {
						uint2 t;
						if(ASMLD) asm volatile("ld.shared.v2.u32 {%0, %1}, [%2];" : "=r"(t.x), "=r"(t.y) : "r"(sbase + addr));
						else t = *reinterpret_cast<const uint2*>(tbl + addr);
						acc[s][k][0] ^= t.x;
						acc[s][k][V - 1] ^= t.y;
					} else {
						uint32_t t;
						if(ASMLD) asm volatile("ld.shared.u32 %0, [%1];" : "=r"(t) : "r"(sbase + addr));
						else t = *reinterpret_cast<const uint32_t*>(tbl + addr);
						acc[s][k][0] ^= t;
					}
				}
			}
		}
	};
	bool ok = true;
	for(unsigned g = 0; g < G && ok; g += 2) {
		if(!mbar_wait(&bars[0], (g >> 1) & 1)) { ok = false; break; }
		lookups(0);
		__syncwarp();
		if(lane == 0) mbar_arrive(&bars[2]);
		if(g + 1 >= G) break;
		if(!mbar_wait(&bars[1], (g >> 1) & 1)) { ok = false; break; }
		lookups(1);
		__syncwarp();
		if(lane == 0) mbar_arrive(&bars[3]);
	}
	if(!ok) return;

#pragma unroll
	for(int s = 0; s < RPW; s++) {
		const unsigned r = rbase + warp * RPW + s;
		if(r < R && laneIn) {
#pragma unroll
			for(int c = 0; c < V; c++) {
				uint32_t v = acc[s][15][c];
#pragma unroll
				for(int k = 14; k >= 0; k--) v = mul2x2(v) ^ acc[s][k][c];
				uint32_t* p = reinterpret_cast<uint32_t*>(rec + (size_t)r * recPitch + colWord) + c;
				if(accumulate) v ^= *p;
				*p = v;
			}
		}
	}
}

template<int RPW, int NL, int WIDE, bool ASMLD>
static int launch_comb_ws(const uint16_t* in, size_t inPitch, unsigned nIn, const uint4* idx, uint16_t* rec,
                          size_t recPitch, unsigned R, size_t nWords, int accumulate, cudaStream_t st)
{
	constexpr int RT = RPW * NL;
	constexpr int V = WIDE ? 2 : 1;
	const size_t smem = 65536 * V + 2 * RT * sizeof(uint4) + 4 * sizeof(uint64_t);
	P2C_CUDA_TRY(cudaFuncSetAttribute(k_comb_ws<RPW, NL, WIDE, ASMLD>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
	const unsigned G = (nIn + 7) / 8;
	const size_t TW = P2C_TILE_WORDS * V;
	dim3 grid((unsigned)((nWords + TW - 1) / TW), (R + RT - 1) / RT);
	k_comb_ws<RPW, NL, WIDE, ASMLD><<<grid, (NL + 4) * 32, smem, st>>>(in, inPitch, nIn, idx, G, rec, recPitch, R, accumulate,
	                                                                 round_up(nWords, P2C_TILE_WORDS));
	P2C_CUDA_TRY(cudaGetLastError());
	return 0;
}

// ---------------------------------------------------------------------------
// Paired-table form: each ring slot holds GP tables (GP consecutive 8-input
// groups, table t at +t*64 KiB, so both reads of a (row, k) pair share the
// PRMT-built address form and differ in the LDS immediate).  With GP = 2 the
// two lookups of a (row, k) pair fold into one three-input XOR
//     P[r][k] ^= T_2s[ idx[r][2s][k] ] ^ T_2s+1[ idx[r][2s+1][k] ]
// so a lookup costs one LDS, one PRMT and half a LOP3 (the one-table forms
// spend a full LOP3 per lookup; the ALU pipe runs at half the LSU rate in
// warp instructions, so the XOR count matters as much as the LDS count).
// Builders prefetch the next slot's inputs and index rows into registers
// before waiting for the slot's buffer to drain.  Waits are bounded as in
// k_comb_ws.
// One work unit (word tile x RT recovery rows, all inputs) of the paired
// form.  Slots are numbered globally from gs0 so that a persistent CTA keeps
// its mbarrier phases running from unit to unit.  Returns false when a
// bounded wait gave up (g_comb_error is set); the thread then does no more
// work in this unit but still returns normally.
template<int RPW, int NL, int GP, int ROLE = 0>   // ROLE: 0 = by warp index, 1 = builder, 2 = lookup
__device__ __forceinline__ bool pair_unit(
	const uint16_t* __restrict__ in, size_t inPitch, unsigned nIn,
	const uint4* __restrict__ idx, unsigned G,
	uint16_t* __restrict__ rec, size_t recPitch, unsigned R, int accumulate,
	size_t tile, unsigned rbase, unsigned gs0, uint8_t* smem)
{
	static_assert(GP == 1 || GP == 2, "one or two tables per slot");
	constexpr int RT = RPW * NL;
	constexpr int TBL = 65536;                         // 256 rows x 256 B (two ring buffers interleaved)
	constexpr int NJ = (RT * GP + 127) / 128;          // index rows staged per builder thread
	uint8_t* tbl = smem;
	uint4* idxs = reinterpret_cast<uint4*>(smem + GP * TBL);                  // [2][GP][RT]
	uint64_t* bars = reinterpret_cast<uint64_t*>(smem + GP * TBL + 2 * GP * RT * sizeof(uint4)); // full[2], empty[2]

	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const size_t colWord = tile * P2C_TILE_WORDS + lane * 2;
	const unsigned NS = (G + GP - 1) / GP;             // ring slots of this unit

	if(ROLE != 2 && (ROLE == 1 || warp >= NL)) {
		// ---------------- builders: 4 warps x 4 high nibbles of each table
		const int bw = warp - NL;
		const int bt = threadIdx.x - NL * 32; // 0..127
		uint32_t x[GP][8];
		uint4 ip[NJ];
		auto fetch = [&](unsigned s) {
#pragma unroll
			for(int t = 0; t < GP; t++)
#pragma unroll
				for(int u = 0; u < 8; u++) {
					const unsigned i = (s * GP + t) * 8 + u;
					x[t][u] = i < nIn ? __ldg(reinterpret_cast<const uint32_t*>(in + (size_t)i * inPitch + colWord)) : 0u;
				}
#pragma unroll
			for(int q = 0; q < NJ; q++) {
				const int jj = bt + q * 128;           // jj = t * RT + j
				ip[q] = make_uint4(0, 0, 0, 0);
				if(jj < GP * RT) {
					const int t = jj / RT, j = jj - t * RT;
					const unsigned g = s * GP + t, r = rbase + j;
					if(g < G && r < R) ip[q] = __ldg(idx + (size_t)r * G + g);
				}
			}
		};
		if(NS) fetch(0);
		for(unsigned s = 0; s < NS; s++) {
			const unsigned gs = gs0 + s;
			const int b = gs & 1;
			if(gs >= 2 && !mbar_wait(&bars[2 + b], ((gs >> 1) - 1) & 1)) return false;
#pragma unroll
			for(int t = 0; t < GP; t++) {
				uint8_t* base = tbl + t * TBL + b * 128 + lane * 4;
#pragma unroll
				for(int hh = 0; hh < 4; hh++) {
					const int h = bw * 4 + hh;
					uint32_t v = 0;
#pragma unroll
					for(int u = 0; u < 4; u++) if(h >> u & 1) v ^= x[t][4 + u];
					uint8_t* rowp = base + h * 16 * 256;
					*reinterpret_cast<uint32_t*>(rowp) = v;
#pragma unroll
					for(int n = 1; n < 16; n++) {
						const int gray = n ^ (n >> 1);
						const int bit = (n & 1) ? 0 : (n & 2) ? 1 : (n & 4) ? 2 : 3;
						v ^= x[t][bit];
						*reinterpret_cast<uint32_t*>(rowp + gray * 256) = v;
					}
				}
			}
#pragma unroll
			for(int q = 0; q < NJ; q++) {
				const int jj = bt + q * 128;
				if(jj < GP * RT) idxs[b * GP * RT + jj] = ip[q];
			}
			mbar_arrive(&bars[b]);  // release: this thread's table rows and index rows
			if(s + 1 < NS) fetch(s + 1);
		}
		return true;
	}

	if constexpr(ROLE == 1) {
		return true;
	} else {
		// ---------------- lookups
		uint32_t acc[RPW][16];
#pragma unroll
		for(int s = 0; s < RPW; s++)
#pragma unroll
			for(int k = 0; k < 16; k++) acc[s][k] = 0;
		const uint32_t lwb = (uint32_t)lane * 4;

		for(unsigned sl = 0; sl < NS; sl++) {
			const unsigned gs = gs0 + sl;
			const int b = gs & 1;
			if(!mbar_wait(&bars[b], (gs >> 1) & 1)) return false;
			const uint32_t lw = lwb + b * 128;
#pragma unroll
			for(int s = 0; s < RPW; s++) {
				const int j = warp * RPW + s;
				if(rbase + j < R) {
					uint32_t qq[GP][4];
#pragma unroll
					for(int t = 0; t < GP; t++) {
						const uint4 q = idxs[(b * GP + t) * RT + j];
						qq[t][0] = q.x; qq[t][1] = q.y; qq[t][2] = q.z; qq[t][3] = q.w;
					}
#pragma unroll
					for(int k = 0; k < 16; k++) {
						// byte0 <- lw.byte0, byte1 <- q.byte(k&3), bytes 2,3 <- lw.byte1 (= 0)
						const uint32_t sel = 4u | ((uint32_t)(k & 3) << 4) | (5u << 8) | (5u << 12);
						uint32_t v = *reinterpret_cast<const uint32_t*>(tbl + __byte_perm(qq[0][k >> 2], lw, sel));
						if(GP == 2) v ^= *reinterpret_cast<const uint32_t*>(tbl + TBL + __byte_perm(qq[GP - 1][k >> 2], lw, sel));
						acc[s][k] ^= v;
					}
				}
			}
			__syncwarp();
			if(lane == 0) mbar_arrive(&bars[2 + b]);
		}

#pragma unroll
		for(int s = 0; s < RPW; s++) {
			const unsigned r = rbase + warp * RPW + s;
			if(r < R) {
				uint32_t v = acc[s][15];
#pragma unroll
				for(int k = 14; k >= 0; k--) v = mul2x2(v) ^ acc[s][k];
				uint32_t* p = reinterpret_cast<uint32_t*>(rec + (size_t)r * recPitch + colWord);
				if(accumulate) v ^= *p;
				*p = v;
			}
		}
		return true;
	}
}

template<int RPW, int NL, int GP>
__device__ __forceinline__ void pair_init_bars(uint8_t* smem) {
	constexpr int RT = RPW * NL;
	uint64_t* bars = reinterpret_cast<uint64_t*>(smem + GP * 65536 + 2 * GP * RT * sizeof(uint4));
	if(threadIdx.x == 0) {
		mbar_init(&bars[0], 128);
		mbar_init(&bars[1], 128);
		mbar_init(&bars[2], NL);
		mbar_init(&bars[3], NL);
	}
}

template<int RPW, int NL, int GP>
__global__ void __launch_bounds__((NL + 4) * 32, 1) k_comb_pair(
	const uint16_t* __restrict__ in, size_t inPitch, unsigned nIn,
	const uint4* __restrict__ idx, unsigned G,
	uint16_t* __restrict__ rec, size_t recPitch, unsigned R, int accumulate)
{
	extern __shared__ __align__(16) uint8_t smem[];
	pair_init_bars<RPW, NL, GP>(smem);
	__syncthreads();
	// one-dimensional grid, recovery blocks fastest: the CTAs that read the
	// same input tile run at the same time and share it through L2
	const unsigned rblocks = (R + RPW * NL - 1) / (RPW * NL);
	const size_t tile = blockIdx.x / rblocks;
	const unsigned rb = blockIdx.x - (unsigned)tile * rblocks;
	pair_unit<RPW, NL, GP>(in, inPitch, nIn, idx, G, rec, recPitch, R, accumulate, tile, rb * (RPW * NL), 0u, smem);
}

// Paired kernel with register reallocation: the builder warpgroup gives up
// registers (setmaxnreg.dec to RB) and the lookup warpgroups take them
// (setmaxnreg.inc to RL), so a lookup warp can hold more recovery rows' P
// accumulators (more rows per CTA share each table build).  The two roles are
// separate branches from the start, each with its own register limit.  The
// host launches it only when the launch's register pool covers the split.
template<int RPW, int NL, int GP, int RL, int RB>
__global__ void __launch_bounds__((NL + 4) * 32, 1) k_comb_pair_rr(
	const uint16_t* __restrict__ in, size_t inPitch, unsigned nIn,
	const uint4* __restrict__ idx, unsigned G,
	uint16_t* __restrict__ rec, size_t recPitch, unsigned R, int accumulate)
{
	static_assert(NL % 4 == 0, "lookup warps form whole warpgroups");
	extern __shared__ __align__(16) uint8_t smem[];
	pair_init_bars<RPW, NL, GP>(smem);
	__syncthreads();
	const unsigned rblocks = (R + RPW * NL - 1) / (RPW * NL);
	const size_t tile = blockIdx.x / rblocks;
	const unsigned rb = blockIdx.x - (unsigned)tile * rblocks;
	if((threadIdx.x >> 5) >= NL) {
		asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" :: "n"(RB));
		pair_unit<RPW, NL, GP, 1>(in, inPitch, nIn, idx, G, rec, recPitch, R, accumulate, tile, rb * (RPW * NL), 0u, smem);
	} else {
		asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" :: "n"(RL));
		pair_unit<RPW, NL, GP, 2>(in, inPitch, nIn, idx, G, rec, recPitch, R, accumulate, tile, rb * (RPW * NL), 0u, smem);
	}
}

// Persistent batched form of the paired kernel: one CTA per SM takes (job,
// word tile, recovery block) units from an atomic ticket.  The builder warps
// own the ticket and run ahead across unit boundaries: every ring slot
// carries a small descriptor (job, recovery block, word tile, row count,
// first/last flags, or the end marker), so the lookup warps start a unit's
// accumulators at its first slot and write its recovery words after its last
// slot, and no CTA-wide barrier separates units.  Unit-boundary latency is
// hidden on the builder side: the job table (up to 64 jobs) is cached in
// shared memory, the next ticket is taken one unit ahead, and the next
// unit's first inputs are fetched while the current unit's last slot is
// consumed.  All waits are bounded: a builder whose wait gave up stops doing
// work and the builder group leaves together at its next group barrier;
// lookup warps stop at their next wait.
struct SlotMeta { unsigned long long tile; unsigned job, rbase, flags, R; };
enum { SLOT_FIRST = 1u, SLOT_LAST = 2u, SLOT_END = 4u };
struct UnitRef { unsigned long long tile; unsigned job, rbase, end, pad; };
constexpr int BATCH_CACHED_JOBS = 64;

__device__ __forceinline__ void builders_sync() { asm volatile("bar.sync 1, 128;" ::: "memory"); }

template<int RPW, int NL, int GP>
__global__ void __launch_bounds__((NL + 4) * 32, 1) k_comb_pair_batched(
	const BatchJob* __restrict__ jobs, unsigned nJobs, unsigned long long totalUnits,
	unsigned long long* __restrict__ counter)
{
	static_assert(GP == 1 || GP == 2, "one or two tables per slot");
	constexpr int RT = RPW * NL;
	constexpr int TBL = 65536;
	constexpr int NJ = (RT * GP + 127) / 128;
	extern __shared__ __align__(16) uint8_t smem[];
	uint8_t* tbl = smem;
	uint4* idxs = reinterpret_cast<uint4*>(smem + GP * TBL);                  // [2][GP][RT]
	uint64_t* bars = reinterpret_cast<uint64_t*>(smem + GP * TBL + 2 * GP * RT * sizeof(uint4));
	__shared__ SlotMeta meta[2];
	__shared__ UnitRef s_unit[2];
	__shared__ BatchJob s_jobs[BATCH_CACHED_JOBS];
	__shared__ int s_babort;

	const bool cached = nJobs <= BATCH_CACHED_JOBS;
	pair_init_bars<RPW, NL, GP>(smem);
	if(threadIdx.x == 0) s_babort = 0;
	if(cached)
		for(unsigned j = threadIdx.x; j < nJobs; j += blockDim.x) s_jobs[j] = jobs[j];
	__syncthreads();
	const BatchJob* JT = cached ? s_jobs : jobs;
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

	if(warp >= NL) {
		// ---------------- builders (4 warps, 128 threads)
		const int bw = warp - NL;
		const int bt = threadIdx.x - NL * 32;
		auto decode = [&](unsigned long long u) {
			UnitRef r;
			r.pad = 0;
			if(u >= totalUnits) { r.end = 1; r.job = 0; r.tile = 0; r.rbase = 0; return r; }
			unsigned lo = 0, hi = nJobs;
			while(hi - lo > 1) {
				const unsigned mid = (lo + hi) >> 1;
				if(JT[mid].unitBase <= u) lo = mid; else hi = mid;
			}
			const unsigned rblocks = (JT[lo].R + RT - 1) / RT;
			const unsigned long long local = u - JT[lo].unitBase;
			r.end = 0; r.job = lo; r.tile = local / rblocks; r.rbase = (unsigned)(local % rblocks) * RT;
			return r;
		};
		unsigned long long tnext = 0;
		if(bt == 0) {
			s_unit[0] = decode(atomicAdd(counter, 1ull));
			tnext = atomicAdd(counter, 1ull);
		}
		builders_sync();
		UnitRef cur = s_unit[0], nxt = cur;

		uint32_t x[GP][8];
		uint4 ip[NJ];
		auto fetch = [&](const UnitRef& ur, unsigned s) {
			const BatchJob& J = JT[ur.job];
			const unsigned nIn = J.nIn, R = J.R, G = (nIn + 7) / 8;
			const size_t colWord = (size_t)ur.tile * P2C_TILE_WORDS + lane * 2;
#pragma unroll
			for(int t = 0; t < GP; t++)
#pragma unroll
				for(int v = 0; v < 8; v++) {
					const unsigned i = (s * GP + t) * 8 + v;
					x[t][v] = i < nIn ? __ldg(reinterpret_cast<const uint32_t*>(J.in + (size_t)i * J.inPitch + colWord)) : 0u;
				}
#pragma unroll
			for(int q = 0; q < NJ; q++) {
				const int jj = bt + q * 128;
				ip[q] = make_uint4(0, 0, 0, 0);
				if(jj < GP * RT) {
					const int t = jj / RT, j = jj - t * RT;
					const unsigned g = s * GP + t, r = ur.rbase + j;
					if(g < G && r < R) ip[q] = __ldg(J.idx + (size_t)r * G + g);
				}
			}
		};

		unsigned gs = 0;
		bool dead = false, prefetched = false;
		for(unsigned k = 0;; ++k) {
			if(cur.end) {                       // end marker slot
				const int b = gs & 1;
				if(dead || (gs >= 2 && !mbar_wait(&bars[2 + b], ((gs >> 1) - 1) & 1))) return;
				if(bt == 0) meta[b].flags = SLOT_END;
				mbar_arrive(&bars[b]);
				return;
			}
			const unsigned R = JT[cur.job].R;
			const unsigned G = (JT[cur.job].nIn + 7) / 8;
			const unsigned NS = G ? (G + GP - 1) / GP : 1;   // a job without inputs sends one zero slot
			if(!dead && !prefetched) fetch(cur, 0);
			prefetched = false;
			for(unsigned s = 0; s < NS; s++) {
				const int b = gs & 1;
				if(!dead && gs >= 2 && !mbar_wait(&bars[2 + b], ((gs >> 1) - 1) & 1)) { dead = true; s_babort = 1; }
				if(!dead) {
#pragma unroll
					for(int t = 0; t < GP; t++) {
						uint8_t* base = tbl + t * TBL + b * 128 + lane * 4;
#pragma unroll
						for(int hh = 0; hh < 4; hh++) {
							const int h = bw * 4 + hh;
							uint32_t v = 0;
#pragma unroll
							for(int w = 0; w < 4; w++) if(h >> w & 1) v ^= x[t][4 + w];
							uint8_t* rowp = base + h * 16 * 256;
							*reinterpret_cast<uint32_t*>(rowp) = v;
#pragma unroll
							for(int n = 1; n < 16; n++) {
								const int gray = n ^ (n >> 1);
								const int bit = (n & 1) ? 0 : (n & 2) ? 1 : (n & 4) ? 2 : 3;
								v ^= x[t][bit];
								*reinterpret_cast<uint32_t*>(rowp + gray * 256) = v;
							}
						}
					}
#pragma unroll
					for(int q = 0; q < NJ; q++) {
						const int jj = bt + q * 128;
						if(jj < GP * RT) idxs[b * GP * RT + jj] = ip[q];
					}
					if(bt == 0) {
						SlotMeta m;
						m.tile = cur.tile; m.job = cur.job; m.rbase = cur.rbase; m.R = R;
						m.flags = (s == 0 ? SLOT_FIRST : 0u) | (s + 1 == NS ? SLOT_LAST : 0u);
						meta[b] = m;
					}
					mbar_arrive(&bars[b]);
				}
				++gs;
				if(s == 0) {
					// publish the next unit (its ticket was taken one unit ago)
					if(bt == 0) {
						s_unit[(k + 1) & 1] = decode(tnext);
						if(tnext < totalUnits) tnext = atomicAdd(counter, 1ull);
					}
					builders_sync();
					if(s_babort) return;
					nxt = s_unit[(k + 1) & 1];
				}
				if(dead) continue;
				if(s + 1 < NS) fetch(cur, s + 1);
				else if(!nxt.end) { fetch(nxt, 0); prefetched = true; }
			}
			cur = nxt;
		}
	}

	// ---------------- lookups
	uint32_t acc[RPW][16];
#pragma unroll
	for(int s = 0; s < RPW; s++)
#pragma unroll
		for(int k = 0; k < 16; k++) acc[s][k] = 0;
	const uint32_t lwb = (uint32_t)lane * 4;
	for(unsigned gs = 0;; ++gs) {
		const int b = gs & 1;
		if(!mbar_wait(&bars[b], (gs >> 1) & 1)) return;
		// only the flags are live during the lookups; the rest of the slot
		// descriptor is read after them, before the slot is released
		const unsigned flags = meta[b].flags;
		if(flags & SLOT_END) return;
		if(flags & SLOT_FIRST) {
#pragma unroll
			for(int s = 0; s < RPW; s++)
#pragma unroll
				for(int k = 0; k < 16; k++) acc[s][k] = 0;
		}
		const uint32_t lw = lwb + b * 128;
		// no per-row guard: rows past R have zero index rows (staged by the
		// builders), so their lookups read table row 0 (= 0)
#pragma unroll
		for(int s = 0; s < RPW; s++) {
			const int j = warp * RPW + s;
			uint32_t qq[GP][4];
#pragma unroll
			for(int t = 0; t < GP; t++) {
				const uint4 q = idxs[(b * GP + t) * RT + j];
				qq[t][0] = q.x; qq[t][1] = q.y; qq[t][2] = q.z; qq[t][3] = q.w;
			}
#pragma unroll
			for(int k = 0; k < 16; k++) {
				const uint32_t sel = 4u | ((uint32_t)(k & 3) << 4) | (5u << 8) | (5u << 12);
				uint32_t v = *reinterpret_cast<const uint32_t*>(tbl + __byte_perm(qq[0][k >> 2], lw, sel));
				if(GP == 2) v ^= *reinterpret_cast<const uint32_t*>(tbl + TBL + __byte_perm(qq[GP - 1][k >> 2], lw, sel));
				acc[s][k] ^= v;
			}
		}
		SlotMeta m = {};
		if(flags & SLOT_LAST) m = meta[b];
		__syncwarp();
		if(lane == 0) mbar_arrive(&bars[2 + b]);   // slot (tables, index rows, descriptor) released
		if(flags & SLOT_LAST) {
			const BatchJob& J = JT[m.job];
			const size_t colWord = (size_t)m.tile * P2C_TILE_WORDS + lane * 2;
#pragma unroll
			for(int s = 0; s < RPW; s++) {
				const unsigned r = m.rbase + warp * RPW + s;
				if(r < m.R) {
					uint32_t v = acc[s][15];
#pragma unroll
					for(int k = 14; k >= 0; k--) v = mul2x2(v) ^ acc[s][k];
					uint32_t* p = reinterpret_cast<uint32_t*>(J.rec + (size_t)r * J.recPitch + colWord);
					if(J.accumulate) v ^= *p;
					*p = v;
				}
			}
		}
	}
}

template<int RPW, int NL, int GP>
static int launch_comb_pair(const uint16_t* in, size_t inPitch, unsigned nIn, const uint4* idx, uint16_t* rec,
                            size_t recPitch, unsigned R, size_t nWords, int accumulate, cudaStream_t st)
{
	constexpr int RT = RPW * NL;
	const size_t smem = 65536 * GP + 2 * GP * RT * sizeof(uint4) + 4 * sizeof(uint64_t);
	P2C_CUDA_TRY(cudaFuncSetAttribute(k_comb_pair<RPW, NL, GP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
	const unsigned G = (nIn + 7) / 8;
	const unsigned long long ctas = (unsigned long long)((nWords + P2C_TILE_WORDS - 1) / P2C_TILE_WORDS) * ((R + RT - 1) / RT);
	if(ctas > 0x7FFFFFFFull) { set_error("comb: %llu CTAs exceed the grid limit", ctas); return -1; }
	k_comb_pair<RPW, NL, GP><<<(unsigned)ctas, (NL + 4) * 32, smem, st>>>(in, inPitch, nIn, idx, G, rec, recPitch, R, accumulate);
	P2C_CUDA_TRY(cudaGetLastError());
	return 0;
}

// Launches the register-reallocating kernel when the launch's register pool
// (registers per thread at launch x threads) covers the split and the split
// lowers the builders and raises the lookups; otherwise returns 1 and the
// caller launches another shape.
template<int RPW, int NL, int GP, int RL, int RB>
static int launch_comb_pair_rr(const uint16_t* in, size_t inPitch, unsigned nIn, const uint4* idx, uint16_t* rec,
                               size_t recPitch, unsigned R, size_t nWords, int accumulate, cudaStream_t st)
{
	constexpr int RT = RPW * NL;
	constexpr int THREADS = (NL + 4) * 32;
	cudaFuncAttributes fa;
	P2C_CUDA_TRY(cudaFuncGetAttributes(&fa, k_comb_pair_rr<RPW, NL, GP, RL, RB>));
	if(fa.numRegs < RB || fa.numRegs > RL || fa.numRegs * THREADS < RL * NL * 32 + RB * 128) return 1;
	const size_t smem = 65536 * GP + 2 * GP * RT * sizeof(uint4) + 4 * sizeof(uint64_t);
	P2C_CUDA_TRY(cudaFuncSetAttribute(k_comb_pair_rr<RPW, NL, GP, RL, RB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
	const unsigned G = (nIn + 7) / 8;
	const unsigned long long ctas = (unsigned long long)((nWords + P2C_TILE_WORDS - 1) / P2C_TILE_WORDS) * ((R + RT - 1) / RT);
	if(ctas > 0x7FFFFFFFull) { set_error("comb: %llu CTAs exceed the grid limit", ctas); return -1; }
	k_comb_pair_rr<RPW, NL, GP, RL, RB><<<(unsigned)ctas, THREADS, smem, st>>>(in, inPitch, nIn, idx, G, rec, recPitch, R,
	                                                                         accumulate);
	P2C_CUDA_TRY(cudaGetLastError());
	return 0;
}

template<int RPW, int NL, int GP>
static int launch_pair_batched(const BatchJob* jobs, unsigned nJobs, unsigned long long totalUnits,
                               unsigned long long* counter, cudaStream_t st)
{
	constexpr int RT = RPW * NL;
	const size_t smem = 65536 * GP + 2 * GP * RT * sizeof(uint4) + 4 * sizeof(uint64_t);
	P2C_CUDA_TRY(cudaFuncSetAttribute(k_comb_pair_batched<RPW, NL, GP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
	int dev = 0, sms = 0;
	P2C_CUDA_TRY(cudaGetDevice(&dev));
	P2C_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
	int occ = 1;
	P2C_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_comb_pair_batched<RPW, NL, GP>, (NL + 4) * 32, smem));
	if(occ < 1) occ = 1;
	unsigned grid = (unsigned)std::min<unsigned long long>((unsigned long long)sms * occ, totalUnits);
	if(!grid) return 0;
	P2C_CUDA_TRY(cudaMemsetAsync(counter, 0, sizeof(unsigned long long), st));
	k_comb_pair_batched<RPW, NL, GP><<<grid, (NL + 4) * 32, smem, st>>>(jobs, nJobs, totalUnits, counter);
	P2C_CUDA_TRY(cudaGetLastError());
	return 0;
}

int comb_error_take() {
	unsigned v = 0, z = 0;
	if(cudaMemcpyFromSymbol(&v, g_comb_error, sizeof(v)) != cudaSuccess) return -1;
	if(v) cudaMemcpyToSymbol(g_comb_error, &z, sizeof(z));
	return (int)v;
}

static std::atomic<int> g_comb_shape{0};
int set_comb_shape(int shape) { return g_comb_shape.exchange(shape); }

// Automatic CTA shape from R (measured on 2000 x 1 MiB, 2000 x 2 MiB and
// 4096 x 256 KiB jobs): above 8 rows the paired-table kernel wins even with
// padded rows (R = 16: 2.1 T vs 1.8 T word mul-adds/s for the best narrow
// shape).  Candidates, with their measured rate per row relative to the
// 72-row block: 72 rows (6 rows x 12 lookup warps, 1.00), 64 rows (8 x 8,
// 0.97) and 96 rows (8 x 12 with register reallocation, 1.018); the one with
// the lowest padded-rows / rate wins above 72 rows.  Up to 8 rows a
// single-warp one-phase CTA builds its own tables.
int comb_auto_shape(unsigned R) {
	if(R <= 8) return 1;
	if(R <= 72) return 16;   // one block either way: measured faster than 64-row blocks at R = 16, 32, 64
	static const struct { int shape; unsigned rows; double rate; } cand[3] = {{16, 72, 1.0}, {18, 64, 0.97}, {28, 96, 1.018}};
	int best = 16;
	double bestCost = 1e300;
	for(const auto& c : cand) {
		const double cost = (double)((R + c.rows - 1) / c.rows * c.rows) / c.rate;
		if(cost < bestCost) { bestCost = cost; best = c.shape; }
	}
	return best;
}

int comb_shape_for(unsigned R) {
	const int s = g_comb_shape.load();
	return s > 0 ? s : comb_auto_shape(R);
}

// Chooses the CTA shape from R: full 96-row blocks for large R, fewer warps /
// rows per warp for small R so that little of a block is wasted.
int comb_muladd(const uint16_t* in, size_t inPitch, unsigned nIn, const uint4* idx, uint16_t* rec, size_t recPitch,
                unsigned R, size_t nWords, int accumulate, int shape, cudaStream_t st)
{
	if(!R || !nWords) return 0;
	if(!nIn) {
		if(!accumulate) P2C_CUDA_TRY(cudaMemset2DAsync(rec, recPitch * 2, 0, nWords * 2, R, st));
		return 0;
	}
	if(shape <= 0) shape = g_comb_shape.load();
	if(shape <= 0) shape = comb_auto_shape(R);
	switch(shape) {
	case 1: return launch_comb<8, 1>(in, inPitch, nIn, idx, rec, recPitch, R, nWords, accumulate, st);
	case 2: return launch_comb<8, 4>(in, inPitch, nIn, idx, rec, recPitch, R, nWords, accumulate, st);
	case 3: return launch_comb<8, 8>(in, inPitch, nIn, idx, rec, recPitch, R, nWords, accumulate, st);
	case 5: return launch_comb<4, 20>(in, inPitch, nIn, idx, rec, recPitch, R, nWords, accumulate, st);
	case 6: return launch_comb<6, 14>(in, inPitch, nIn, idx, rec, recPitch, R, nWords, accumulate, st);
	case 7: return launch_comb<5, 16>(in, inPitch, nIn, idx, rec, recPitch, R, nWords, accumulate, st);
	case 8: return launch_comb<4, 16>(in, inPitch, nIn, idx, rec, recPitch, R, nWords, accumulate, st);
	case 9: return launch_comb<2, 32>(in, inPitch, nIn, idx, rec, recPitch, R, nWords, accumulate, st);
	case 10: return launch_comb_ws<8, 8, 0, false>(in, inPitch, nIn, idx, rec, recPitch, R, nWords, accumulate, st);
	case 11: return launch_comb_ws<6, 12, 0, false>(in, inPitch, nIn, idx, rec, recPitch, R, nWords, accumulate, st);
	case 12: return launch_comb_ws<5, 12, 0, false>(in, inPitch, nIn, idx, rec, recPitch, R, nWords, accumulate, st);
	case 13: return launch_comb_ws<6, 12, 0, true>(in, inPitch, nIn, idx, rec, recPitch, R, nWords, accumulate, st);
	case 14: return launch_comb_ws<3, 12, 1, false>(in, inPitch, nIn, idx, rec, recPitch, R, nWords, accumulate, st);
	case 15: return launch_comb_ws<4, 8, 1, false>(in, inPitch, nIn, idx, rec, recPitch, R, nWords, accumulate, st);
	case 16: return launch_comb_pair<6, 12, 2>(in, inPitch, nIn, idx, rec, recPitch, R, nWords, accumulate, st);
	case 17: return launch_comb_pair<5, 12, 2>(in, inPitch, nIn, idx, rec, recPitch, R, nWords, accumulate, st);
	case 18: return launch_comb_pair<8, 8, 2>(in, inPitch, nIn, idx, rec, recPitch, R, nWords, accumulate, st);
	case 19: return launch_comb_pair<7, 10, 2>(in, inPitch, nIn, idx, rec, recPitch, R, nWords, accumulate, st);
	case 20: return launch_comb_pair<6, 12, 1>(in, inPitch, nIn, idx, rec, recPitch, R, nWords, accumulate, st);
	case 21: return launch_comb_pair<4, 16, 2>(in, inPitch, nIn, idx, rec, recPitch, R, nWords, accumulate, st);
	case 22: return launch_comb_pair<3, 20, 2>(in, inPitch, nIn, idx, rec, recPitch, R, nWords, accumulate, st);
	case 23: return launch_comb_pair<8, 4, 2>(in, inPitch, nIn, idx, rec, recPitch, R, nWords, accumulate, st);
	case 24: return launch_comb_pair<8, 2, 2>(in, inPitch, nIn, idx, rec, recPitch, R, nWords, accumulate, st);
	case 25: return launch_comb_pair<8, 1, 2>(in, inPitch, nIn, idx, rec, recPitch, R, nWords, accumulate, st);
	case 26: case 27: case 28: {
		int rc = shape == 26 ? launch_comb_pair_rr<7, 12, 2, 144, 56>(in, inPitch, nIn, idx, rec, recPitch, R, nWords, accumulate, st)
		       : shape == 27 ? launch_comb_pair_rr<6, 12, 2, 152, 56>(in, inPitch, nIn, idx, rec, recPitch, R, nWords, accumulate, st)
		       : launch_comb_pair_rr<8, 12, 2, 152, 56>(in, inPitch, nIn, idx, rec, recPitch, R, nWords, accumulate, st);
		if(rc != 1) return rc;
		return launch_comb_pair<6, 12, 2>(in, inPitch, nIn, idx, rec, recPitch, R, nWords, accumulate, st);
	}
	default: return launch_comb<8, 12>(in, inPitch, nIn, idx, rec, recPitch, R, nWords, accumulate, st);
	}
}

// recovery rows per CTA of the persistent batched shapes: 1..4 one-phase
// (8 rows per warp x 1, 4, 8, 12 warps), 5..7 paired (72, 64, 32 rows)
int batched_rows(int shape) {
	static const int rt[8] = {0, 8, 32, 64, 96, 72, 64, 32};
	return shape >= 1 && shape <= 7 ? rt[shape] : 0;
}

// units per job for a batched shape: word tiles x recovery blocks
unsigned long long comb_units(unsigned R, size_t nWords, int shape) {
	const unsigned RT = (unsigned)batched_rows(shape);
	if(!RT) return 0;
	return (unsigned long long)((nWords + P2C_TILE_WORDS - 1) / P2C_TILE_WORDS) * ((R + RT - 1) / RT);
}

template<int RPW, int NW>
static int launch_batched(const BatchJob* jobs, unsigned nJobs, unsigned long long totalUnits,
                          unsigned long long* counter, int ctasPerSm, cudaStream_t st)
{
	constexpr int RT = RPW * NW;
	const size_t smem = 65536 + 2 * RT * sizeof(uint4);
	P2C_CUDA_TRY(cudaFuncSetAttribute(k_comb_batched<RPW, NW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
	int dev = 0, sms = 0;
	P2C_CUDA_TRY(cudaGetDevice(&dev));
	P2C_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
	int occ = 1;
	P2C_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_comb_batched<RPW, NW>, NW * 32, smem));
	if(ctasPerSm > 0 && ctasPerSm < occ) occ = ctasPerSm;
	if(occ < 1) occ = 1;
	unsigned grid = (unsigned)std::min<unsigned long long>((unsigned long long)sms * occ, totalUnits);
	if(!grid) return 0;
	P2C_CUDA_TRY(cudaMemsetAsync(counter, 0, sizeof(unsigned long long), st));
	k_comb_batched<RPW, NW><<<grid, NW * 32, smem, st>>>(jobs, nJobs, totalUnits, counter);
	P2C_CUDA_TRY(cudaGetLastError());
	return 0;
}

int comb_batched(const BatchJob* dJobs, unsigned nJobs, unsigned long long totalUnits, unsigned long long* dCounter,
                 int shape, cudaStream_t st)
{
	if(!nJobs || !totalUnits) return 0;
	switch(shape) {
	case 1: return launch_batched<8, 1>(dJobs, nJobs, totalUnits, dCounter, 0, st);
	case 2: return launch_batched<8, 4>(dJobs, nJobs, totalUnits, dCounter, 0, st);
	case 3: return launch_batched<8, 8>(dJobs, nJobs, totalUnits, dCounter, 0, st);
	case 4: return launch_batched<8, 12>(dJobs, nJobs, totalUnits, dCounter, 0, st);
	case 5: return launch_pair_batched<6, 12, 2>(dJobs, nJobs, totalUnits, dCounter, st);
	case 6: return launch_pair_batched<8, 8, 2>(dJobs, nJobs, totalUnits, dCounter, st);
	case 7: return launch_pair_batched<8, 4, 2>(dJobs, nJobs, totalUnits, dCounter, st);
	default: set_error("batched comb shape %d not available (1..7)", shape); return -1;
	}
}

} // namespace p2c
