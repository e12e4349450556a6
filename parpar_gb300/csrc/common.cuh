// Shared definitions for the GB300 PAR2 recovery engine (sm_103a).
//
// Data model (all little-endian 16-bit GF(2^16) words, polynomial 0x1100B):
//   a "row" holds one slice chunk of S bytes (S even), zero-padded to
//   Sp = roundup(S, 8) bytes, followed by one 8-byte checksum block (four
//   16-bit lanes), i.e. rowWords = (Sp + 8) / 2 words.  Rows are stored
//   `pitch` words apart, pitch a multiple of 64 words (128 bytes), so every
//   row starts 128-byte aligned and every 64-word tile is in bounds.
#pragma once
#include <cstddef>
#include <cstdint>
#include <algorithm>
#include <cuda_runtime.h>

#define P2C_POLY 0x1100Bu
#define P2C_TILE_WORDS 64
#define P2C_CKSUM_BYTES 8

namespace p2c {

inline size_t round_up(size_t v, size_t m) { return (v + m - 1) / m * m; }
__device__ __forceinline__ size_t round_up_dev(size_t v, size_t m) { return (v + m - 1) / m * m; }
// words in a row: padded data + checksum block
inline size_t row_words(size_t sliceBytes) { return (round_up(sliceBytes, 8) + P2C_CKSUM_BYTES) / 2; }
inline size_t row_pitch(size_t sliceBytes) { return round_up(row_words(sliceBytes), P2C_TILE_WORDS); }

// multiply both 16-bit halves of v by 2 (x) in GF(2^16)
__device__ __forceinline__ uint32_t mul2x2(uint32_t v) {
	uint32_t hi = (v >> 15) & 0x00010001u;
	return ((v << 1) & 0xFFFEFFFEu) ^ (hi * (P2C_POLY & 0xFFFFu));
}
__device__ __forceinline__ uint64_t mul2x4(uint64_t v) {
	const uint64_t m = 0x0001000100010001ull;
	return ((v << 1) & ~m) ^ (((v >> 15) & m) * (uint64_t)(P2C_POLY & 0xFFFFu));
}

// device-resident antilog / log tables (2 x 65535 entries of exp for
// wrap-free index sums, 65536 of log), uploaded once per device
struct GfTables {
	const uint16_t* exp;  // exp[e] = 2^e, e in [0, 131070)
	const uint16_t* log;  // log[x], log[0] unused
	const uint16_t* inLog; // PAR2 input logs for inputs 0..32767
};

__device__ __forceinline__ uint16_t gf_mul_tab(const GfTables& t, uint16_t a, uint16_t b) {
	if(!a || !b) return 0;
	return t.exp[(uint32_t)t.log[a] + t.log[b]];
}

// per-lane multiply of a 4-lane checksum block by 2^e
__device__ __forceinline__ uint64_t cksum_mul_exp(const GfTables& t, uint64_t ck, uint32_t e) {
	uint64_t r = 0;
	uint32_t em = e % 65535u;
#pragma unroll
	for(int l = 0; l < 4; l++) {
		uint16_t v = (uint16_t)(ck >> (16 * l));
		uint16_t p = v ? t.exp[(uint32_t)t.log[v] + em] : 0;
		r |= (uint64_t)p << (16 * l);
	}
	return r;
}

} // namespace p2c

// error plumbing shared by the host-side files
namespace p2c {
void set_error(const char* fmt, ...);
const char* get_error();
}

// On failure the message is recorded and the runtime's per-thread "last
// error" is consumed, so that a non-sticky failure (e.g. an allocation that
// does not fit) is not reported again by the next launch check.
#define P2C_CUDA_TRY(expr) do { cudaError_t _e = (expr); if(_e != cudaSuccess) { \
	(void)cudaGetLastError(); \
	p2c::set_error("%s:%d %s: %s", __FILE__, __LINE__, #expr, cudaGetErrorString(_e)); return -1; } } while(0)
