// Two further multiply-accumulate variants with the comb kernel's contract
// (rec[r] (^)= sum_i c(r,i) in[i] over nWords words), kept for comparison and
// for the autotuner:
//
//  * xor    — the bit-sliced (16 bit planes) formulation of the reference's XOR
//             bit-dependency method (gf16/gf16_xor_*.c, xor_depends/info.md):
//             the coefficient's 16x16 GF(2) matrix applied to 16 input planes
//             with predicated XORs; no tables, bound by the integer pipe.
//  * nibble — split-nibble tables (the OpenCL LOOKUP idea,
//             gf16/controller_ocl_init.cpp:112-253, with 4 x 16-entry tables per
//             coefficient instead of 2 x 256): c*x = T0[x&15]^T1[x>>4&15]^
//             T2[x>>8&15]^T3[x>>12], tables built per CTA in shared memory.
#include "common.cuh"
#include "kernels.h"

namespace p2c {

// ---------------------------------------------------- xor over 16 bit planes
// The bit-sliced form of the XOR bit-dependency method: 32 words are held as
// 16 bit planes (plane b = bit b of each of the 32 words), and multiplying by
// c maps the 16 input planes to 16 output planes through c's 16x16 GF(2)
// matrix (column b = c * x^b): out[j] ^= in[b] wherever bit j of c*x^b is set.
//
// Warp: 32 recovery rows, one per lane; every lane sees the same input planes
// (built with 16 warp ballots per 32 words, no shared memory), so the planes
// of an input are made once and serve 32 rows.  Each lane walks the 256 bits
// of its own coefficient's matrix: a mask per bit (all ones where the bit is
// set) and one three-input LOP3, acc ^= plane & mask, per group of 32 words
// (PG groups per warp = 32*PG words), i.e. about (2 + PG) / (32 PG) * 256
// integer ops per word mul-add — the matrix is data, so the network of XORs
// cannot be fixed at compile time as the reference's per-coefficient JIT does.
// At the end each lane turns its 16 output planes back into words with an
// in-register bit transpose.
#define P2C_PG 4
__device__ __forceinline__ void bit_transpose16(uint32_t (&m)[16]) {
	// m[k] holds a 16-bit row k; afterwards m[k] bit b = old m[b] bit k
#pragma unroll
	for(int k = 0; k < 8; k++) { uint32_t t = ((m[k] >> 8) ^ m[k + 8]) & 0x00FFu; m[k] ^= t << 8; m[k + 8] ^= t; }
#pragma unroll
	for(int k = 0; k < 16; k++) if((k & 4) == 0 && k < 12) { uint32_t t = ((m[k] >> 4) ^ m[k + 4]) & 0x0F0Fu; m[k] ^= t << 4; m[k + 4] ^= t; }
#pragma unroll
	for(int k = 0; k < 16; k++) if((k & 2) == 0 && k < 14) { uint32_t t = ((m[k] >> 2) ^ m[k + 2]) & 0x3333u; m[k] ^= t << 2; m[k + 2] ^= t; }
#pragma unroll
	for(int k = 0; k < 16; k += 2) { uint32_t t = ((m[k] >> 1) ^ m[k + 1]) & 0x5555u; m[k] ^= t << 1; m[k + 1] ^= t; }
}

__global__ void __launch_bounds__(128) k_xor_planes(
	const uint16_t* __restrict__ in, size_t inPitch, unsigned nIn, const uint16_t* __restrict__ coeff,
	uint16_t* __restrict__ rec, size_t recPitch, unsigned R, size_t nWords, int accumulate)
{
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const unsigned r = blockIdx.y * 128 + warp * 32 + lane;
	const size_t w0 = (size_t)blockIdx.x * (32 * P2C_PG);
	if(blockIdx.y * 128 + warp * 32 >= R) return;          // whole warp past the last row
	const bool rowOk = r < R;
	uint32_t acc[16][P2C_PG];
#pragma unroll
	for(int j = 0; j < 16; j++)
#pragma unroll
		for(int g = 0; g < P2C_PG; g++) acc[j][g] = 0;
	const uint16_t* crow = coeff + (size_t)(rowOk ? r : 0) * nIn;
	for(unsigned i = 0; i < nIn; i++) {
		// planes of the 32*PG words of input i (word 32g + lane in lane `lane`)
		uint32_t pl[16][P2C_PG];
		const uint16_t* src = in + (size_t)i * inPitch + w0;
#pragma unroll
		for(int g = 0; g < P2C_PG; g++) {
			const size_t w = w0 + 32 * g + lane;
			const uint32_t x = w < nWords ? (uint32_t)__ldg(src + 32 * g + lane) : 0u;
#pragma unroll
			for(int b = 0; b < 16; b++) {
				// all 32 lanes vote here, outside any lane-dependent control flow
				uint32_t v;
				asm volatile("{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %1, 0;\n\tvote.sync.ballot.b32 %0, q, 0xffffffff;\n\t}"
				             : "=r"(v) : "r"((x >> b) & 1u));
				pl[b][g] = v;
			}
		}
		uint32_t col = rowOk ? (uint32_t)__ldg(crow + i) : 0u;
#pragma unroll
		for(int b = 0; b < 16; b++) {
#pragma unroll
			for(int j = 0; j < 16; j++) {
				// all-ones when bit j of c*x^b is set: out plane j takes in plane b
				const uint32_t m = (uint32_t)((int32_t)(col << (31 - j)) >> 31);
#pragma unroll
				for(int g = 0; g < P2C_PG; g++) acc[j][g] ^= pl[b][g] & m;   // one LOP3
			}
			// next column: c * x^(b+1)
			col <<= 1;
			col = (col ^ ((col >> 16) * (P2C_POLY & 0xFFFFu))) & 0xFFFFu;
		}
	}
	if(!rowOk) return;
	uint16_t* dst = rec + (size_t)r * recPitch + w0;
#pragma unroll
	for(int g = 0; g < P2C_PG; g++) {
#pragma unroll
		for(int half = 0; half < 2; half++) {
			uint32_t m[16];
#pragma unroll
			for(int j = 0; j < 16; j++) m[j] = (acc[j][g] >> (16 * half)) & 0xFFFFu;
			bit_transpose16(m);          // m[k] = word 32g + 16*half + k
#pragma unroll
			for(int k = 0; k < 16; k += 2) {
				const size_t w = w0 + 32 * g + 16 * half + k;
				if(w >= nWords) continue;
				uint32_t* p = reinterpret_cast<uint32_t*>(dst + 32 * g + 16 * half + k);
				const uint32_t v = m[k] | (m[k + 1] << 16);
				*p = accumulate ? (*p ^ v) : v;
			}
		}
	}
}

int xor_planes_muladd(const uint16_t* in, size_t inPitch, unsigned nIn, const uint16_t* coeff, uint16_t* rec,
                      size_t recPitch, unsigned R, size_t nWords, int accumulate, cudaStream_t st)
{
	if(!R || !nWords) return 0;
	// rows are padded to 64-word multiples: tiles of 128 words stay inside
	// the pitch once nWords is rounded to 128 where the pitch allows it
	const size_t tile = 32 * P2C_PG;
	size_t nw = round_up(nWords, 2);
	if(round_up(nWords, tile) <= inPitch && round_up(nWords, tile) <= recPitch) nw = round_up(nWords, tile);
	dim3 grid((unsigned)((nw + tile - 1) / tile), (R + 127) / 128);
	k_xor_planes<<<grid, 128, 0, st>>>(in, inPitch, nIn, coeff, rec, recPitch, R, nw, accumulate);
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
