// Hashing kernels: per-slice MD5 + CRC32 (the IFSC entries) and per-file MD5,
// one independent hash stream per GPU thread.
//
// Semantics follow the reference's HasherInput (hasher/hasher_base.h:103-186,
// src/gf.cc:926-954, 1015-1039):
//   IFSC entry of a slice = MD5(slice bytes zero-padded to the slice size)
//                           ++ CRC32(same bytes) little-endian      (20 bytes)
//   file MD5 = MD5 of the file's bytes (no padding).
// MD5 is RFC 1321; CRC32 is the reflected IEEE polynomial 0xEDB88320.  The
// zero padding of the CRC is applied by multiplying the register by
// x^(8*pad) mod P (hasher/crc_zeropad.c:55-66); the MD5 must process the
// padding bytes.  The CRC is computed slice-by-4 from shared-memory tables in
// the same thread, in the bubbles of the MD5 dependency chain.
#include "common.cuh"
#include "kernels.h"

namespace p2c {

// RFC 1321 round constants (a constexpr table: indexed by the unrolled step
// number, each becomes an immediate operand).
__device__ constexpr uint32_t c_md5K[64] = {
	0xd76aa478,0xe8c7b756,0x242070db,0xc1bdceee,0xf57c0faf,0x4787c62a,0xa8304613,0xfd469501,
	0x698098d8,0x8b44f7af,0xffff5bb1,0x895cd7be,0x6b901122,0xfd987193,0xa679438e,0x49b40821,
	0xf61e2562,0xc040b340,0x265e5a51,0xe9b6c7aa,0xd62f105d,0x02441453,0xd8a1e681,0xe7d3fbc8,
	0x21e1cde6,0xc33707d6,0xf4d50d87,0x455a14ed,0xa9e3e905,0xfcefa3f8,0x676f02d9,0x8d2a4c8a,
	0xfffa3942,0x8771f681,0x6d9d6122,0xfde5380c,0xa4beea44,0x4bdecfa9,0xf6bb4b60,0xbebfbc70,
	0x289b7ec6,0xeaa127fa,0xd4ef3085,0x04881d05,0xd9d4d039,0xe6db99e5,0x1fa27cf8,0xc4ac5665,
	0xf4292244,0x432aff97,0xab9423a7,0xfc93a039,0x655b59c3,0x8f0ccc92,0xffeff47d,0x85845dd1,
	0x6fa87e4f,0xfe2ce6e0,0xa3014314,0x4e0811a1,0xf7537e82,0xbd3af235,0x2ad7d2bb,0xeb86d391};

__device__ __forceinline__ uint32_t rotl(uint32_t x, int s) { return __funnelshift_l(x, x, s); }

// one 64-byte block; m[16] little-endian words
__device__ __forceinline__ void md5_block(uint32_t st[4], const uint32_t m[16]) {
	uint32_t a = st[0], b = st[1], c = st[2], d = st[3];
#pragma unroll
	for(int i = 0; i < 64; i++) {
		uint32_t f; int g, s;
		if(i < 16) { f = d ^ (b & (c ^ d)); g = i; s = (i & 3) == 0 ? 7 : (i & 3) == 1 ? 12 : (i & 3) == 2 ? 17 : 22; }
		else if(i < 32) { f = c ^ (d & (b ^ c)); g = (5 * i + 1) & 15; s = (i & 3) == 0 ? 5 : (i & 3) == 1 ? 9 : (i & 3) == 2 ? 14 : 20; }
		else if(i < 48) { f = b ^ c ^ d; g = (3 * i + 5) & 15; s = (i & 3) == 0 ? 4 : (i & 3) == 1 ? 11 : (i & 3) == 2 ? 16 : 23; }
		else { f = c ^ (b | ~d); g = (7 * i) & 15; s = (i & 3) == 0 ? 6 : (i & 3) == 1 ? 10 : (i & 3) == 2 ? 15 : 21; }
		// a + K + m does not depend on the previous step; the add of f is the
		// only add on the step's dependency chain (LOP3 -> add -> rotate-add).
		// It is written as its own PTX add so that the compiler cannot fold f
		// into the off-chain sum: with the four terms in one C expression the
		// step compiled to a second dependent add and ran ~21 cycles instead
		// of ~17 on GB300 with message words loaded from memory.
		const uint32_t pre = a + c_md5K[i] + m[g];
		uint32_t t;
		asm("add.u32 %0, %1, %2;" : "=r"(t) : "r"(f), "r"(pre));
		a = d; d = c; c = b;
		b = b + rotl(t, s);
	}
	st[0] += a; st[1] += b; st[2] += c; st[3] += d;
}

struct CrcTabs;
__device__ __forceinline__ uint32_t crc_word(const CrcTabs& T, uint32_t crc, uint32_t w);
struct NoTabs {};
__device__ __forceinline__ uint32_t crc_word(const NoTabs&, uint32_t crc, uint32_t) { return crc; }

__device__ __forceinline__ void load_block(const uint4* p4, size_t b, uint32_t m[16]) {
#pragma unroll
	for(int q = 0; q < 4; q++) {
		uint4 v = __ldg(p4 + b * 4 + q);
		m[4 * q] = v.x; m[4 * q + 1] = v.y; m[4 * q + 2] = v.z; m[4 * q + 3] = v.w;
	}
}

// MD5 (and optionally CRC32) over `full` consecutive 64-byte blocks with the
// loads software-pipelined two blocks ahead: a single thread walks a long
// serial chain, so without prefetch every block would wait a full memory
// latency.
// L2 prefetch distance (64-byte blocks) ahead of the register prefetch: the
// register loads then mostly hit L2, well inside their two-block lead
#define P2C_MD5_L2_AHEAD 48

template<bool CRC, typename Tabs>
__device__ __forceinline__ void md5_blocks(uint32_t st[4], uint32_t& crc, const Tabs& T, const uint4* p4, size_t full) {
	uint32_t A[16], B[16];
	if(full > 0) load_block(p4, 0, A);
	if(full > 1) load_block(p4, 1, B);
	for(size_t b = 0; b < full; b += 2) {
		uint32_t m[16];
		// one 128-byte line (two blocks) per iteration, only inside this row
		if(b + P2C_MD5_L2_AHEAD < full)
			asm volatile("prefetch.global.L2 [%0];" :: "l"(p4 + (b + P2C_MD5_L2_AHEAD) * 4));
#pragma unroll
		for(int q = 0; q < 16; q++) m[q] = A[q];
		if(b + 2 < full) load_block(p4, b + 2, A);
		if(CRC) {
#pragma unroll
			for(int q = 0; q < 16; q++) crc = crc_word(T, crc, m[q]);
		}
		md5_block(st, m);
		if(b + 1 < full) {
#pragma unroll
			for(int q = 0; q < 16; q++) m[q] = B[q];
			if(b + 3 < full) load_block(p4, b + 3, B);
			if(CRC) {
#pragma unroll
				for(int q = 0; q < 16; q++) crc = crc_word(T, crc, m[q]);
			}
			md5_block(st, m);
		}
	}
}

// The same for a stream whose 64-byte blocks start at a 4-byte (not 16-byte)
// boundary of memory: 32-bit loads, same two-block register pipeline and L2
// prefetch.
__device__ __forceinline__ void load_block32(const uint32_t* p, size_t b, uint32_t m[16]) {
#pragma unroll
	for(int q = 0; q < 16; q++) m[q] = __ldg(p + b * 16 + q);
}
__device__ __forceinline__ void md5_blocks32(uint32_t st[4], const uint32_t* p, size_t full) {
	uint32_t A[16], B[16];
	if(full > 0) load_block32(p, 0, A);
	if(full > 1) load_block32(p, 1, B);
	for(size_t b = 0; b < full; b += 2) {
		uint32_t m[16];
		if(b + P2C_MD5_L2_AHEAD < full)
			asm volatile("prefetch.global.L2 [%0];" :: "l"(p + (b + P2C_MD5_L2_AHEAD) * 16));
#pragma unroll
		for(int q = 0; q < 16; q++) m[q] = A[q];
		if(b + 2 < full) load_block32(p, b + 2, A);
		md5_block(st, m);
		if(b + 1 < full) {
#pragma unroll
			for(int q = 0; q < 16; q++) m[q] = B[q];
			if(b + 3 < full) load_block32(p, b + 3, B);
			md5_block(st, m);
		}
	}
}

// CRC32 slice-by-4 tables, built per CTA in shared memory
struct CrcTabs { uint32_t t[4][256]; };

__device__ void crc_tabs_build(CrcTabs& T) {
	for(int i = threadIdx.x; i < 256; i += blockDim.x) {
		uint32_t c = i;
		for(int k = 0; k < 8; k++) c = (c >> 1) ^ (0xEDB88320u & (0u - (c & 1)));
		T.t[0][i] = c;
	}
	__syncthreads();
	for(int i = threadIdx.x; i < 256; i += blockDim.x) {
		uint32_t c = T.t[0][i];
		for(int j = 1; j < 4; j++) { c = (c >> 8) ^ T.t[0][c & 255]; T.t[j][i] = c; }
	}
	__syncthreads();
}

__device__ __forceinline__ uint32_t crc_word(const CrcTabs& T, uint32_t crc, uint32_t w) {
	crc ^= w;
	return T.t[3][crc & 255] ^ T.t[2][(crc >> 8) & 255] ^ T.t[1][(crc >> 16) & 255] ^ T.t[0][crc >> 24];
}
__device__ __forceinline__ uint32_t crc_byte(const CrcTabs& T, uint32_t crc, uint32_t b) {
	return (crc >> 8) ^ T.t[0][(crc ^ b) & 255];
}
// a*b mod P, reflected bit order (bit 31 = x^0)
__device__ uint32_t crc_mulmod(uint32_t a, uint32_t b) {
	uint32_t r = 0;
	for(int i = 0; i < 32; i++) {
		r ^= (0u - (b >> 31)) & a;
		b <<= 1;
		a = (a >> 1) ^ (0xEDB88320u & (0u - (a & 1)));
	}
	return r;
}
// raw register after `n` more zero bytes: multiply by x^(8n)
__device__ uint32_t crc_zero_extend(uint32_t reg, uint64_t n) {
	uint32_t xn = 0x00800000u; // x^8
	while(n) {
		if(n & 1) reg = crc_mulmod(reg, xn);
		xn = crc_mulmod(xn, xn);
		n >>= 1;
	}
	return reg;
}

// MD5 finish for a stream whose unprocessed tail (< 64 bytes) is in `tail`
// (little-endian words, bytes beyond tailLen zero) with `zeros` zero bytes
// still to append, then the standard padding (md5_final_block semantics,
// hasher/md5-final.c:4-60).
__device__ void md5_finish(uint32_t st[4], uint32_t tail[16], uint32_t tailLen, uint64_t zeros, uint64_t total) {
	// zero padding: fill the current block, then whole zero blocks
	if(tailLen + zeros >= 64) {
		md5_block(st, tail); // bytes past tailLen are zero already
		zeros -= 64 - tailLen;
		uint32_t z[16];
#pragma unroll
		for(int i = 0; i < 16; i++) z[i] = 0;
		for(uint64_t b = zeros / 64; b; b--) md5_block(st, z);
		zeros %= 64;
#pragma unroll
		for(int i = 0; i < 16; i++) tail[i] = 0;
		tailLen = 0;
	}
	tailLen += (uint32_t)zeros;
	// 0x80 terminator
	tail[tailLen >> 2] |= 0x80u << (8 * (tailLen & 3));
	tailLen++;
	if(tailLen > 56) {
		md5_block(st, tail);
#pragma unroll
		for(int i = 0; i < 16; i++) tail[i] = 0;
	}
	const uint64_t bits = total << 3;
	tail[14] = (uint32_t)bits;
	tail[15] = (uint32_t)(bits >> 32);
	md5_block(st, tail);
}

__device__ __forceinline__ void md5_init(uint32_t st[4]) {
	st[0] = 0x67452301u; st[1] = 0xefcdab89u; st[2] = 0x98badcfeu; st[3] = 0x10325476u;
}

// ---- per-slice MD5 + CRC32 --------------------------------------------------
// one thread per row: row i holds lens[i] bytes (or sliceBytes), hashed as if
// zero-padded to sliceBytes.  out: 20 bytes per row.
__global__ void __launch_bounds__(128) k_slice_hash(const uint8_t* rows, size_t pitch, unsigned n,
                                                   const uint32_t* lens, size_t sliceBytes, uint8_t* out)
{
	__shared__ CrcTabs T;
	crc_tabs_build(T);
	const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= n) return;
	const size_t len = lens ? min((size_t)lens[i], sliceBytes) : sliceBytes;
	const uint8_t* p = rows + (size_t)i * pitch;
	uint32_t st[4];
	md5_init(st);
	uint32_t crc = 0xFFFFFFFFu;
	const size_t full = len / 64;
	md5_blocks<true>(st, crc, T, reinterpret_cast<const uint4*>(p), full);
	// tail bytes
	uint32_t tail[16];
#pragma unroll
	for(int q = 0; q < 16; q++) tail[q] = 0;
	const uint32_t rem = (uint32_t)(len - full * 64);
	for(uint32_t k = 0; k < rem; k++) {
		uint32_t byte = p[full * 64 + k];
		tail[k >> 2] |= byte << (8 * (k & 3));
		crc = crc_byte(T, crc, byte);
	}
	md5_finish(st, tail, rem, sliceBytes - len, sliceBytes);
	crc = ~crc_zero_extend(crc, sliceBytes - len);
	uint8_t* o = out + (size_t)i * 20;
#pragma unroll
	for(int w = 0; w < 4; w++) {
		o[4 * w] = (uint8_t)st[w]; o[4 * w + 1] = (uint8_t)(st[w] >> 8);
		o[4 * w + 2] = (uint8_t)(st[w] >> 16); o[4 * w + 3] = (uint8_t)(st[w] >> 24);
	}
	o[16] = (uint8_t)crc; o[17] = (uint8_t)(crc >> 8); o[18] = (uint8_t)(crc >> 16); o[19] = (uint8_t)(crc >> 24);
}

int slice_hash(const void* rows, size_t pitchBytes, unsigned n, const uint32_t* dLens, size_t sliceBytes,
               uint8_t* dOut, cudaStream_t st)
{
	if(!n) return 0;
	if(pitchBytes % 16) { set_error("row pitch must be a multiple of 16 bytes"); return -1; }
	k_slice_hash<<<(n + 127) / 128, 128, 0, st>>>((const uint8_t*)rows, pitchBytes, n, dLens, sliceBytes, dOut);
	P2C_CUDA_TRY(cudaGetLastError());
	return 0;
}

// ---- calibration: the MD5 dependency-chain bound ------------------------------
// One MD5 stream on one GPU thread is bound by the latency of its serial
// step chain (3 dependent integer ops per step: the round function, the add
// of a + K + m, the rotate-and-add), not by memory.  This kernel runs that
// chain on register-resident data, one warp on one SM: the bytes/s of one
// lane is the ceiling for the per-file and per-slice hash kernels.  The state
// carries across blocks, so no block's work can be hoisted.
__global__ void __launch_bounds__(32) k_md5_chain(uint32_t* sink, unsigned blocks) {
	uint32_t st[4] = {0x67452301u ^ threadIdx.x, 0xefcdab89u, 0x98badcfeu, 0x10325476u};
	// the same message block every time, held in registers: each step's
	// a + K + m term has nothing to wait for, so the loop runs at the step
	// chain's own latency (LOP3 -> add -> rotate-add)
	uint32_t m[16];
#pragma unroll
	for(int q = 0; q < 16; q++) m[q] = (uint32_t)(q + 1) * 0x9E3779B9u ^ threadIdx.x;
	for(unsigned b = 0; b < blocks; b++) md5_block(st, m);
	if((st[0] ^ st[1] ^ st[2] ^ st[3]) == 0x5EEDF00Du && blocks == 0) sink[threadIdx.x] = st[0];
}

int md5_chain_rate(double* bytesPerSec, cudaStream_t st) {
	const unsigned blocks = 40000;   // ~25 ms at ~100 MB/s
	cudaEvent_t e0, e1;
	P2C_CUDA_TRY(cudaEventCreate(&e0));
	P2C_CUDA_TRY(cudaEventCreate(&e1));
	k_md5_chain<<<1, 32, 0, st>>>(nullptr, blocks / 8); // warm-up
	float best = 0.f;
	for(int rep = 0; rep < 3; rep++) {
		cudaEventRecord(e0, st);
		k_md5_chain<<<1, 32, 0, st>>>(nullptr, blocks);
		cudaEventRecord(e1, st);
		cudaError_t e = cudaEventSynchronize(e1);
		if(e != cudaSuccess) {
			cudaEventDestroy(e0); cudaEventDestroy(e1);
			set_error("md5 chain calibration: %s", cudaGetErrorString(e));
			return -1;
		}
		float ms = 0.f;
		cudaEventElapsedTime(&ms, e0, e1);
		if(rep == 0 || ms < best) best = ms;
	}
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	P2C_CUDA_TRY(cudaGetLastError());
	*bytesPerSec = best > 0.f ? 64.0 * blocks / (best * 1e-3) : 0.0;
	return 0;
}

// ---- per-file MD5 -----------------------------------------------------------
// file f = rows first[f] .. first[f]+ceil(len[f]/sliceBytes)-1, each row
// contributing sliceBytes bytes except the last.  One thread per file.
template<int MAXT>
__global__ void __launch_bounds__(MAXT) k_file_md5(const uint8_t* rows, size_t pitch, unsigned nFiles,
                                                   const uint64_t* fileLen, const uint32_t* firstRow,
                                                   size_t sliceBytes, uint8_t* out)
{
	const unsigned f = blockIdx.x * blockDim.x + threadIdx.x;
	if(f >= nFiles) return;
	const uint64_t total = fileLen[f];
	uint32_t st[4];
	md5_init(st);
	uint32_t tail[16];
#pragma unroll
	for(int q = 0; q < 16; q++) tail[q] = 0;
	uint32_t tailLen = 0;
	uint64_t done = 0;
	size_t row = firstRow[f];
	while(done < total) {
		const size_t take = (size_t)min((uint64_t)sliceBytes, total - done);
		const uint8_t* p = rows + row * pitch;
		size_t pos = 0;
		if(tailLen == 0 && (sliceBytes % 64) == 0) {
			// block-aligned fast path
			const size_t full = take / 64;
			uint32_t nocrc = 0;
			md5_blocks<false>(st, nocrc, NoTabs{}, reinterpret_cast<const uint4*>(p), full);
			pos = full * 64;
		}
		for(; pos < take; pos++) {
			tail[tailLen >> 2] |= (uint32_t)p[pos] << (8 * (tailLen & 3));
			if(++tailLen == 64) {
				md5_block(st, tail);
#pragma unroll
				for(int q = 0; q < 16; q++) tail[q] = 0;
				tailLen = 0;
			}
		}
		done += take;
		row++;
	}
	md5_finish(st, tail, tailLen, 0, total);
	uint8_t* o = out + (size_t)f * 16;
#pragma unroll
	for(int w = 0; w < 4; w++) {
		o[4 * w] = (uint8_t)st[w]; o[4 * w + 1] = (uint8_t)(st[w] >> 8);
		o[4 * w + 2] = (uint8_t)(st[w] >> 16); o[4 * w + 3] = (uint8_t)(st[w] >> 24);
	}
}

int file_md5(const void* rows, size_t pitchBytes, unsigned nFiles, const uint64_t* dFileLen, const uint32_t* dFirstRow,
             size_t sliceBytes, uint8_t* dOut, cudaStream_t st, unsigned filesPerBlock)
{
	if(!nFiles) return 0;
	if(pitchBytes % 16) { set_error("row pitch must be a multiple of 16 bytes"); return -1; }
	// one thread per file.  filesPerBlock 1 (default): one file per block,
	// spread over SMs (the fastest chains: 108 MB/s).  32: one warp of files
	// per block, ~6 % slower per chain but ceil(nFiles/32) blocks instead of
	// nFiles, each of which keeps a full-register-file CTA of other work off
	// its SM while the chains run.  Up to 512: the files of several jobs on
	// as few SMs as possible (a warp issues one instruction per ~4-cycle
	// dependency step, so a few warps per scheduler do not slow each other).
	if(filesPerBlock == 1) {
		k_file_md5<32><<<nFiles, 1, 0, st>>>((const uint8_t*)rows, pitchBytes, nFiles, dFileLen, dFirstRow, sliceBytes, dOut);
	} else if(filesPerBlock == 32) {
		k_file_md5<32><<<(nFiles + 31) / 32, 32, 0, st>>>((const uint8_t*)rows, pitchBytes, nFiles, dFileLen, dFirstRow,
		                                                   sliceBytes, dOut);
	} else {
		if(filesPerBlock % 32 || filesPerBlock > 512) {
			set_error("files per block %u must be 1 or a multiple of 32 up to 512", filesPerBlock);
			return -1;
		}
		const unsigned per = min(filesPerBlock, (nFiles + 31) / 32 * 32);
		k_file_md5<512><<<(nFiles + per - 1) / per, per, 0, st>>>((const uint8_t*)rows, pitchBytes, nFiles, dFileLen,
		                                                             dFirstRow, sliceBytes, dOut);
	}
	P2C_CUDA_TRY(cudaGetLastError());
	return 0;
}

// ---- per-file MD5 with the bytes staged through shared memory --------------
// One thread per file, as above, but the thread does not load its bytes from
// global memory itself: it keeps P2C_STG_NS bulk asynchronous copies
// (cp.async.bulk, the TMA engine) of P2C_STG_CH-byte chunks of its file in
// flight into its own ring of shared memory, each completing on an mbarrier
// of the ring, and hashes from shared memory.  The chain then never waits on
// an L2 miss, whatever else the GPU runs (another job's contraction streaming
// gigabytes through L2 evicted the prefetched lines of the register-loading
// kernel).  Needs sliceBytes % 64 == 0 (chunks never split an MD5 block) and
// 16-byte aligned rows; every wait is bounded (on timeout the error flag is
// set and the chain stops; its digest is then not valid).
#define P2C_STG_CH 1024
#define P2C_STG_NS 3
#define P2C_STG_STRIDE (P2C_STG_CH * P2C_STG_NS + 16)
#define P2C_STG_WAIT (1u << 24)
__device__ unsigned g_hash_error;

__device__ __forceinline__ uint32_t hs_saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool hs_wait(uint32_t bar, uint32_t parity) {
	for(unsigned i = 0; i < P2C_STG_WAIT; i++) {
		uint32_t ok;
		asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
		             : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
		if(ok) return true;
	}
	return false;
}

template<int NT>
__global__ void __launch_bounds__(NT) k_file_md5_staged(const uint8_t* __restrict__ rows, size_t pitch, unsigned nFiles,
                                                        const uint64_t* __restrict__ fileLen,
                                                        const uint32_t* __restrict__ firstRow, size_t sliceBytes,
                                                        uint8_t* __restrict__ out, const uint32_t* __restrict__ outIndex)
{
	extern __shared__ __align__(128) uint8_t smem[];
	const unsigned t = threadIdx.x;
	const unsigned f = blockIdx.x * NT + t;
	uint8_t* ring = smem + (size_t)t * P2C_STG_STRIDE;
	uint64_t* bars = reinterpret_cast<uint64_t*>(smem + (size_t)NT * P2C_STG_STRIDE) + t * P2C_STG_NS;
	const uint32_t ringA = hs_saddr(ring), barA = hs_saddr(bars);
	for(int k = 0; k < P2C_STG_NS; k++)
		asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(barA + 8 * k) : "memory");
	asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	__syncthreads();
	if(f >= nFiles) return;

	const uint64_t total = fileLen[f];
	const uint8_t* base = rows + (size_t)firstRow[f] * pitch;
	// chunk cursor: row r of the file, byte offset `off` inside it
	size_t issR = 0, issOff = 0;
	uint64_t issLeft = total;          // file bytes from the issue cursor on
	auto issue = [&](int slot) -> uint32_t {
		const uint64_t rowBytes = issLeft + issOff < sliceBytes ? issLeft + issOff : sliceBytes;
		const uint32_t size = (uint32_t)min((uint64_t)P2C_STG_CH, rowBytes - issOff);
		const uint32_t csize = (size + 15u) & ~15u;
		const uint8_t* src = base + issR * pitch + issOff;
		const uint32_t bar = barA + 8 * slot;
		asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}"
		             :: "r"(bar), "r"(csize) : "memory");
		asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
		             :: "r"(ringA + slot * P2C_STG_CH), "l"(src), "r"(csize), "r"(bar) : "memory");
		issLeft -= size;
		issOff += size;
		if(issOff == rowBytes) { issR++; issOff = 0; }
		return size;
	};
	uint32_t sizes[P2C_STG_NS];
	uint32_t phase = 0;                // bit k: parity of slot k's next completion
	uint32_t pend = 0;                 // bit k: slot k has a copy in flight
	int inflight = 0;
#pragma unroll
	for(int k = 0; k < P2C_STG_NS; k++) {
		sizes[k] = 0;
		if(issLeft) { sizes[k] = issue(k); inflight++; pend |= 1u << k; }
	}
	uint32_t st[4];
	md5_init(st);
	uint32_t tail[16];
#pragma unroll
	for(int q = 0; q < 16; q++) tail[q] = 0;
	uint32_t tailLen = 0;
	bool ok = true;
	for(int slot = 0; inflight > 0; slot = slot + 1 == P2C_STG_NS ? 0 : slot + 1) {
		if(!hs_wait(barA + 8 * slot, (phase >> slot) & 1u)) { ok = false; break; }
		phase ^= 1u << slot;
		pend &= ~(1u << slot);
		inflight--;
		uint32_t size = 0;
#pragma unroll
		for(int k = 0; k < P2C_STG_NS; k++) if(k == slot) size = sizes[k];
		const uint4* p4 = reinterpret_cast<const uint4*>(ring + slot * P2C_STG_CH);
		const uint32_t full = size / 64;
		uint32_t A[16];
		if(full) {
#pragma unroll
			for(int q = 0; q < 4; q++) { uint4 v = p4[q]; A[4 * q] = v.x; A[4 * q + 1] = v.y; A[4 * q + 2] = v.z; A[4 * q + 3] = v.w; }
		}
		for(uint32_t b = 0; b < full; b++) {
			uint32_t m[16];
#pragma unroll
			for(int q = 0; q < 16; q++) m[q] = A[q];
			if(b + 1 < full) {
#pragma unroll
				for(int q = 0; q < 4; q++) {
					uint4 v = p4[(b + 1) * 4 + q];
					A[4 * q] = v.x; A[4 * q + 1] = v.y; A[4 * q + 2] = v.z; A[4 * q + 3] = v.w;
				}
			}
			md5_block(st, m);
		}
		if(size % 64) {   // only the file's last chunk: its partial block goes to the finish
			const uint8_t* pb = ring + slot * P2C_STG_CH + full * 64;
			for(uint32_t k = 0; k < size % 64; k++) tail[k >> 2] |= (uint32_t)pb[k] << (8 * (k & 3));
			tailLen = size % 64;
		}
		if(issLeft) {
			// order this thread's reads of the slot before the copy that reuses it
			asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
#pragma unroll
			for(int k = 0; k < P2C_STG_NS; k++) if(k == slot) sizes[k] = issue(slot);
			inflight++;
			pend |= 1u << slot;
		}
	}
	if(!ok) {
		atomicExch(&g_hash_error, 1u);
		// let this chain's copies still in flight land before the block exits
		for(int k = 0; k < P2C_STG_NS; k++)
			if(pend >> k & 1u) hs_wait(barA + 8 * k, (phase >> k) & 1u);
		return;
	}
	md5_finish(st, tail, tailLen, 0, total);
	uint8_t* o = out + (size_t)(outIndex ? outIndex[f] : f) * 16;
#pragma unroll
	for(int w = 0; w < 4; w++) {
		o[4 * w] = (uint8_t)st[w]; o[4 * w + 1] = (uint8_t)(st[w] >> 8);
		o[4 * w + 2] = (uint8_t)(st[w] >> 16); o[4 * w + 3] = (uint8_t)(st[w] >> 24);
	}
}

int file_md5_staged(const void* rows, size_t pitchBytes, unsigned nFiles, const uint64_t* dFileLen,
                    const uint32_t* dFirstRow, size_t sliceBytes, uint8_t* dOut, unsigned filesPerBlock, cudaStream_t st,
                    const uint32_t* dOutIndex)
{
	if(!nFiles) return 0;
	if(pitchBytes % 16 || ((uintptr_t)rows & 15)) { set_error("staged file MD5: rows must be 16-byte aligned"); return -1; }
	if(sliceBytes % 64 || !sliceBytes) { set_error("staged file MD5: slice size must be a multiple of 64 bytes"); return -1; }
	if(filesPerBlock != 32 && filesPerBlock != 64) { set_error("staged file MD5: 32 or 64 files per block"); return -1; }
	const size_t smem = (size_t)filesPerBlock * (P2C_STG_STRIDE + 8 * P2C_STG_NS);
	if(filesPerBlock == 32) {
		P2C_CUDA_TRY(cudaFuncSetAttribute(k_file_md5_staged<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
		k_file_md5_staged<32><<<(nFiles + 31) / 32, 32, smem, st>>>((const uint8_t*)rows, pitchBytes, nFiles, dFileLen,
		                                                             dFirstRow, sliceBytes, dOut, dOutIndex);
	} else {
		P2C_CUDA_TRY(cudaFuncSetAttribute(k_file_md5_staged<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
		k_file_md5_staged<64><<<(nFiles + 63) / 64, 64, smem, st>>>((const uint8_t*)rows, pitchBytes, nFiles, dFileLen,
		                                                             dFirstRow, sliceBytes, dOut, dOutIndex);
	}
	P2C_CUDA_TRY(cudaGetLastError());
	return 0;
}

int hash_error_take() {
	unsigned v = 0, z = 0;
	if(cudaMemcpyFromSymbol(&v, g_hash_error, sizeof(v)) != cudaSuccess) return -1;
	if(v) cudaMemcpyToSymbol(g_hash_error, &z, sizeof(z));
	return (int)v;
}

// ---- MD5 of equal-length rows (recovery packets; MD5Multi, hasher/hasher.h:33-56)
// row i: prefix[i] (prefixLen bytes, host-assembled packet header) followed by
// dataLen bytes of row data.  One thread per row.
__global__ void __launch_bounds__(128) k_rows_md5(const uint8_t* rows, size_t pitch, unsigned n, size_t dataLen,
                                                 const uint8_t* prefix, unsigned prefixLen, uint8_t* out)
{
	const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= n) return;
	uint32_t st[4];
	md5_init(st);
	uint32_t tail[16];
#pragma unroll
	for(int q = 0; q < 16; q++) tail[q] = 0;
	uint32_t tailLen = 0;
	const uint8_t* pre = prefix ? prefix + (size_t)i * prefixLen : nullptr;
	for(unsigned k = 0; k < prefixLen; k++) {
		tail[tailLen >> 2] |= (uint32_t)pre[k] << (8 * (tailLen & 3));
		if(++tailLen == 64) { md5_block(st, tail); for(int q = 0; q < 16; q++) tail[q] = 0; tailLen = 0; }
	}
	const uint8_t* p = rows + (size_t)i * pitch;
	size_t pos = 0;
	if(tailLen == 0) {
		uint32_t nocrc = 0;
		md5_blocks<false>(st, nocrc, NoTabs{}, reinterpret_cast<const uint4*>(p), dataLen / 64);
		pos = dataLen / 64 * 64;
	} else if(tailLen % 4 == 0 && dataLen >= 64 - tailLen) {
		// a prefix of whole words (the 36-byte packet header): complete its
		// block with data words, then the data's blocks start 4-byte aligned
		const uint32_t* d32 = reinterpret_cast<const uint32_t*>(p);
		const unsigned need = (64 - tailLen) / 4;
		for(unsigned q = 0; q < need; q++) tail[(tailLen >> 2) + q] = __ldg(d32 + q);
		md5_block(st, tail);
#pragma unroll
		for(int q = 0; q < 16; q++) tail[q] = 0;
		tailLen = 0;
		pos = (size_t)need * 4;
		const size_t full = (dataLen - pos) / 64;
		md5_blocks32(st, d32 + need, full);
		pos += full * 64;
	}
	for(; pos < dataLen; pos++) {
		tail[tailLen >> 2] |= (uint32_t)p[pos] << (8 * (tailLen & 3));
		if(++tailLen == 64) { md5_block(st, tail); for(int q = 0; q < 16; q++) tail[q] = 0; tailLen = 0; }
	}
	md5_finish(st, tail, tailLen, 0, prefixLen + dataLen);
	uint8_t* o = out + (size_t)i * 16;
#pragma unroll
	for(int w = 0; w < 4; w++) {
		o[4 * w] = (uint8_t)st[w]; o[4 * w + 1] = (uint8_t)(st[w] >> 8);
		o[4 * w + 2] = (uint8_t)(st[w] >> 16); o[4 * w + 3] = (uint8_t)(st[w] >> 24);
	}
}

int rows_md5(const void* rows, size_t pitchBytes, unsigned n, size_t dataLen, const uint8_t* dPrefix, unsigned prefixLen,
             uint8_t* dOut, cudaStream_t st)
{
	if(!n) return 0;
	if(pitchBytes % 16) { set_error("row pitch must be a multiple of 16 bytes"); return -1; }
	k_rows_md5<<<(n + 127) / 128, 128, 0, st>>>((const uint8_t*)rows, pitchBytes, n, dataLen, dPrefix, prefixLen, dOut);
	P2C_CUDA_TRY(cudaGetLastError());
	return 0;
}

} // namespace p2c
