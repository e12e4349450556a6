/*
 * ORACLE — test infrastructure, not product code.
 *
 * A plain-C restatement of the reference's CPU algorithm for the PAR2 recovery
 * path (ParPar, Ravencentric/ParPar).  The CUDA path is tested against it:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * it.  The product library (libpar2cuda.so) never links or calls it.
 *
 * Parity pin: every function below is checked against the reference's own
 * compiled code (oracle/ref.mk -> oracle/_ref/libparref.so, driven by
 * oracle/ref_shim.cpp) through the golden fixtures in tests/golden/, which
 * tests/golden/make_golden.py generates from that build.
 *
 * Contents (reference file:line each function follows):
 *   GF(2^16), polynomial 0x1100B ............ gf16/gf16_global.h:9-10
 *   PAR2 input logs / coefficients .......... gf16/gfmat_coeff.c:6-77
 *   region multiply-accumulate (LOOKUP) ..... gf16/gf16_lookup.c:124-181, 218-249
 *   recovery computation .................... gf16/controller_cpu.cpp:372-385, 463-537
 *   exponent-0 row = XOR of inputs .......... gf16/controller_cpu.cpp:498-512
 *   internal checksum (generic, 8-byte) ..... gf16/gf16_checksum_generic.h:25-130,
 *                                             gf16/gf16_cksum_base.h:13-60
 *   MD5 (RFC 1321) + zero-pad finish ........ hasher/md5-final.c:4-60
 *   CRC32 (reflected 0xEDB88320) + zero pad . hasher/crc_zeropad.c:7-66
 *   IFSC entries / file MD5 ................. hasher/hasher_base.h:103-186
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define OR_POLY 0x1100Bu

static uint16_t or_exp_tab[65536 * 2];
static uint16_t or_log_tab[65536];
static uint16_t or_in_log[32768];
static int or_ready = 0;
static pthread_once_t or_once = PTHREAD_ONCE_INIT;

static void or_build(void) {
	uint32_t n = 1;
	for(uint32_t e = 0; e < 65535; e++) {
		or_exp_tab[e] = (uint16_t)n;
		or_exp_tab[e + 65535] = (uint16_t)n;
		or_log_tab[n] = (uint16_t)e;
		n <<= 1;
		if(n & 0x10000) n ^= OR_POLY;
	}
	or_exp_tab[131070] = or_exp_tab[0];
	or_exp_tab[131071] = or_exp_tab[1];
	or_log_tab[0] = 0;
	/* gfmat_coeff.c:12-22 — input i gets the i-th exponent (counting from 1)
	 * that is not divisible by 3, 5, 17 or 257, i.e. coprime with 65535 */
	uint32_t e = 0;
	for(uint32_t i = 0; i < 32768; i++) {
		do { e++; } while(e % 3 == 0 || e % 5 == 0 || e % 17 == 0 || e % 257 == 0);
		or_in_log[i] = (uint16_t)e;
	}
	or_ready = 1;
}

void or_init(void) { pthread_once(&or_once, or_build); }

/* 2^v for any v (reduced mod 65535) — gf16_exp, gfmat_coeff.c:43-54 */
uint16_t or_exp(uint32_t v) { or_init(); return or_exp_tab[v % 65535u]; }

uint16_t or_mul(uint16_t a, uint16_t b) {
	or_init();
	if(!a || !b) return 0;
	return or_exp_tab[(uint32_t)or_log_tab[a] + or_log_tab[b]];
}

/* shift-and-xor multiply, independent of the tables (cross-check) */
uint16_t or_mul_slow(uint16_t a, uint16_t b) {
	uint32_t p = 0, x = a;
	for(int i = 0; i < 16; i++) {
		if(b >> i & 1) p ^= x;
		x <<= 1;
		if(x & 0x10000) x ^= OR_POLY;
	}
	return (uint16_t)p;
}

uint16_t or_input_log(uint16_t input) { or_init(); return or_in_log[input & 32767]; }

/* gfmat_coeff.c:60-77: coefficient = 2^((log_i * e) mod 65535) */
uint16_t or_coeff_from_log(uint16_t inLog, uint16_t exponent) {
	or_init();
	return or_exp_tab[((uint32_t)inLog * exponent) % 65535u];
}
uint16_t or_coeff(uint16_t input, uint16_t exponent) {
	return or_coeff_from_log(or_input_log(input), exponent);
}

/* Split 8-bit tables for multiply by c: c*x = lo[x & 255] ^ hi[x >> 8]
 * (the LOOKUP method's two 256-entry tables, gf16_lookup.c:124-181). */
static void or_tables(uint16_t c, uint16_t* lo, uint16_t* hi) {
	for(unsigned v = 0; v < 256; v++) {
		lo[v] = or_mul(c, (uint16_t)v);
		hi[v] = or_mul(c, (uint16_t)(v << 8));
	}
}

/* dst[w] ^= c * src[w] over `words` little-endian u16 words */
void or_muladd_region(uint8_t* dst, const uint8_t* src, size_t words, uint16_t c) {
	uint16_t lo[256], hi[256];
	or_init();
	or_tables(c, lo, hi);
	for(size_t w = 0; w < words; w++) {
		uint16_t x = (uint16_t)(src[2 * w] | (src[2 * w + 1] << 8));
		uint16_t y = (uint16_t)(dst[2 * w] | (dst[2 * w + 1] << 8));
		y ^= lo[x & 255] ^ hi[x >> 8];
		dst[2 * w] = (uint8_t)y;
		dst[2 * w + 1] = (uint8_t)(y >> 8);
	}
}

/* ---------- recovery computation (multi-threaded LOOKUP port) ---------- */
typedef struct {
	const uint8_t* inputs; const size_t* lens; const uint16_t* coeffs; /* [r][n] */
	unsigned n, r; size_t slice; uint8_t* out;
	size_t chunk; unsigned nchunks; unsigned nthreads; unsigned tid;
} or_job;

static void* or_worker(void* arg) {
	or_job* j = (or_job*)arg;
	uint16_t* lo = (uint16_t*)malloc(256 * sizeof(uint16_t) * 2);
	uint16_t* hi = lo + 256;
	/* static split of (byte chunk × recovery row) units, as run_kernel does
	 * (controller_cpu.cpp:539-624) */
	size_t units = (size_t)j->nchunks * j->r;
	for(size_t u = j->tid; u < units; u += j->nthreads) {
		unsigned ch = (unsigned)(u / j->r), row = (unsigned)(u % j->r);
		size_t off = (size_t)ch * j->chunk;
		size_t len = j->slice - off < j->chunk ? j->slice - off : j->chunk;
		uint8_t* dst = j->out + (size_t)row * j->slice + off;
		memset(dst, 0, len);
		for(unsigned i = 0; i < j->n; i++) {
			uint16_t c = j->coeffs[(size_t)row * j->n + i];
			size_t have = j->lens[i] > off ? j->lens[i] - off : 0; /* zero padding beyond lens[i] */
			if(have > len) have = len;
			if(!have || !c) continue;
			const uint8_t* src = j->inputs + (size_t)i * j->slice + off;
			or_tables(c, lo, hi);
			size_t w = 0;
			for(; 2 * w + 1 < have; w++) {
				uint16_t x = (uint16_t)(src[2 * w] | (src[2 * w + 1] << 8));
				uint16_t p = lo[x & 255] ^ hi[x >> 8];
				dst[2 * w] ^= (uint8_t)p;
				dst[2 * w + 1] ^= (uint8_t)(p >> 8);
			}
			if(2 * w < have) { /* odd tail byte: high byte is zero padding */
				uint16_t p = lo[src[2 * w]];
				dst[2 * w] ^= (uint8_t)p;
				dst[2 * w + 1] ^= (uint8_t)(p >> 8);
			}
		}
	}
	free(lo);
	return NULL;
}

/* inputs: n rows of `slice` bytes (row i meaningful up to lens[i], zero beyond);
 * coeffs: [r][n]; out: r rows of `slice` bytes.  slice must be even. */
int or_recover_coeffs(const uint8_t* inputs, const size_t* lens, const uint16_t* coeffs,
                      unsigned n, size_t slice, unsigned r, uint8_t* out, int threads) {
	or_init();
	if(slice & 1) return -1;
	if(threads < 1) threads = 1;
	if(threads > 256) threads = 256;
	size_t chunk = 32768;
	if(chunk > slice) chunk = slice;
	unsigned nchunks = (unsigned)((slice + chunk - 1) / chunk);
	pthread_t th[256];
	or_job jobs[256];
	for(int t = 0; t < threads; t++) {
		or_job jb = {inputs, lens, coeffs, n, r, slice, out, chunk, nchunks, (unsigned)threads, (unsigned)t};
		jobs[t] = jb;
	}
	if(threads == 1) { or_worker(&jobs[0]); return 0; }
	for(int t = 0; t < threads; t++) pthread_create(&th[t], NULL, or_worker, &jobs[t]);
	for(int t = 0; t < threads; t++) pthread_join(th[t], NULL);
	return 0;
}

/* PAR2 recovery: coefficients from input numbers and recovery exponents
 * (set_coeffs, controller_cpu.cpp:372-379) */
int or_recover(const uint8_t* inputs, const size_t* lens, const uint16_t* inputNums, unsigned n,
               size_t slice, const uint16_t* exps, unsigned r, uint8_t* out, int threads) {
	or_init();
	uint16_t* coeffs = (uint16_t*)malloc(sizeof(uint16_t) * (size_t)n * r + 2);
	if(!coeffs) return -2;
	for(unsigned row = 0; row < r; row++)
		for(unsigned i = 0; i < n; i++)
			coeffs[(size_t)row * n + i] = or_coeff(inputNums[i], exps[row]);
	int rc = or_recover_coeffs(inputs, lens, coeffs, n, slice, r, out, threads);
	free(coeffs);
	return rc;
}

/* ---------- internal GF checksum, generic 8-byte block (4 u16 lanes) ---------- */
static inline uint64_t or_mul2x4(uint64_t v) {
	const uint64_t m = 0x0001000100010001ULL;
	return ((v << 1) & ~m) ^ (((v >> 15) & m) * (OR_POLY & 0xFFFF));
}
static inline uint64_t or_rd64(const uint8_t* p, size_t avail) {
	uint64_t v = 0;
	for(size_t b = 0; b < 8 && b < avail; b++) v |= (uint64_t)p[b] << (8 * b);
	return v;
}
/* multiply each lane by 2^e (gf16_checksum_exp_generic) */
static uint64_t or_ck_exp(uint64_t ck, uint32_t e) {
	uint16_t c = or_exp(e);
	uint64_t res = 0;
	for(int b = 15; b >= 0; b--) {
		res = or_mul2x4(res);
		if(c >> b & 1) res ^= ck;
	}
	return res;
}
/* Checksum of `srcLen` bytes zero-padded to `sliceLen` (gf16_cksum_copy):
 * Horner over 8-byte blocks, ck = mul2(ck) ^ block, then the zero tail
 * multiplies by 2^(tail blocks). */
uint64_t or_cksum(const uint8_t* src, size_t srcLen, size_t sliceLen) {
	or_init();
	uint64_t ck = 0;
	for(size_t p = 0; p < srcLen; p += 8) ck = or_mul2x4(ck) ^ or_rd64(src + p, srcLen - p);
	size_t done = (srcLen + 7) / 8 * 8;
	if(srcLen < sliceLen && done < sliceLen)
		ck = or_ck_exp(ck, (uint32_t)(((sliceLen - done + 7) / 8) % 65535));
	return ck;
}
/* Verifies `len` bytes against their carried checksum (gf16_cksum_copy_check):
 * rewind by 2^-(blocks), re-run Horner over the data, require zero. */
int or_cksum_check(const uint8_t* data, size_t len, uint64_t ck) {
	or_init();
	uint32_t nb = (uint32_t)(((len + 7) / 8) % 65535);
	ck = or_ck_exp(ck, 65535 - nb);
	for(size_t p = 0; p < len; p += 8) ck = or_mul2x4(ck) ^ or_rd64(data + p, len - p);
	return ck == 0;
}

/* ---------- MD5 (RFC 1321) ---------- */
static const uint32_t or_md5_k[64] = {
	0xd76aa478,0xe8c7b756,0x242070db,0xc1bdceee,0xf57c0faf,0x4787c62a,0xa8304613,0xfd469501,
	0x698098d8,0x8b44f7af,0xffff5bb1,0x895cd7be,0x6b901122,0xfd987193,0xa679438e,0x49b40821,
	0xf61e2562,0xc040b340,0x265e5a51,0xe9b6c7aa,0xd62f105d,0x02441453,0xd8a1e681,0xe7d3fbc8,
	0x21e1cde6,0xc33707d6,0xf4d50d87,0x455a14ed,0xa9e3e905,0xfcefa3f8,0x676f02d9,0x8d2a4c8a,
	0xfffa3942,0x8771f681,0x6d9d6122,0xfde5380c,0xa4beea44,0x4bdecfa9,0xf6bb4b60,0xbebfbc70,
	0x289b7ec6,0xeaa127fa,0xd4ef3085,0x04881d05,0xd9d4d039,0xe6db99e5,0x1fa27cf8,0xc4ac5665,
	0xf4292244,0x432aff97,0xab9423a7,0xfc93a039,0x655b59c3,0x8f0ccc92,0xffeff47d,0x85845dd1,
	0x6fa87e4f,0xfe2ce6e0,0xa3014314,0x4e0811a1,0xf7537e82,0xbd3af235,0x2ad7d2bb,0xeb86d391};
static const uint8_t or_md5_r[64] = {7,12,17,22,7,12,17,22,7,12,17,22,7,12,17,22,5,9,14,20,5,9,14,20,5,9,14,20,5,9,14,20,
	4,11,16,23,4,11,16,23,4,11,16,23,4,11,16,23,6,10,15,21,6,10,15,21,6,10,15,21,6,10,15,21};

static void or_md5_block(uint32_t* st, const uint8_t* blk) {
	uint32_t m[16];
	for(int i = 0; i < 16; i++)
		m[i] = (uint32_t)blk[4*i] | ((uint32_t)blk[4*i+1] << 8) | ((uint32_t)blk[4*i+2] << 16) | ((uint32_t)blk[4*i+3] << 24);
	uint32_t a = st[0], b = st[1], c = st[2], d = st[3];
	/* fully unrolled, so the round constants and rotations fold into the code */
#pragma GCC unroll 64
	for(int i = 0; i < 64; i++) {
		uint32_t f; int g;
		if(i < 16) { f = (b & c) | (~b & d); g = i; }
		else if(i < 32) { f = (d & b) | (~d & c); g = (5 * i + 1) & 15; }
		else if(i < 48) { f = b ^ c ^ d; g = (3 * i + 5) & 15; }
		else { f = c ^ (b | ~d); g = (7 * i) & 15; }
		uint32_t t = a + f + or_md5_k[i] + m[g];
		a = d; d = c; c = b;
		b = b + ((t << or_md5_r[i]) | (t >> (32 - or_md5_r[i])));
	}
	st[0] += a; st[1] += b; st[2] += c; st[3] += d;
}

/* MD5 of data[0..len) followed by zeroPad zero bytes (md5_final_block semantics) */
void or_md5(const uint8_t* data, size_t len, uint64_t zeroPad, uint8_t out[16]) {
	uint32_t st[4] = {0x67452301, 0xefcdab89, 0x98badcfe, 0x10325476};
	uint8_t blk[64];
	uint64_t total = len + zeroPad;
	size_t p = 0;
	for(; p + 64 <= len; p += 64) or_md5_block(st, data + p);
	size_t rem = len - p;
	memcpy(blk, data + p, rem);
	uint64_t pad = zeroPad;
	while(rem + pad >= 64) { /* zero-filled blocks */
		memset(blk + rem, 0, 64 - rem);
		or_md5_block(st, blk);
		pad -= 64 - rem;
		rem = 0;
	}
	memset(blk + rem, 0, 64 - rem);
	rem += (size_t)pad;
	blk[rem++] = 0x80;
	if(rem > 56) { memset(blk + rem, 0, 64 - rem); or_md5_block(st, blk); rem = 0; memset(blk, 0, 64); }
	memset(blk + rem, 0, 56 - rem);
	uint64_t bits = total << 3;
	for(int i = 0; i < 8; i++) blk[56 + i] = (uint8_t)(bits >> (8 * i));
	or_md5_block(st, blk);
	for(int i = 0; i < 4; i++) {
		out[4*i] = (uint8_t)st[i]; out[4*i+1] = (uint8_t)(st[i] >> 8);
		out[4*i+2] = (uint8_t)(st[i] >> 16); out[4*i+3] = (uint8_t)(st[i] >> 24);
	}
}

/* ---------- CRC32 (IEEE, reflected) ---------- */
static uint32_t or_crc_tab[256];
static pthread_once_t or_crc_once = PTHREAD_ONCE_INIT;
static void or_crc_build(void) {
	for(uint32_t i = 0; i < 256; i++) {
		uint32_t c = i;
		for(int k = 0; k < 8; k++) c = (c >> 1) ^ (0xEDB88320u & (0u - (c & 1)));
		or_crc_tab[i] = c;
	}
}
/* a*b mod P in the reflected bit order (bit 31 = x^0) */
static uint32_t or_crc_mulmod(uint32_t a, uint32_t b) {
	uint32_t r = 0;
	for(int i = 0; i < 32; i++) {
		if(b & 0x80000000u) r ^= a;
		b <<= 1;
		a = (a >> 1) ^ (0xEDB88320u & (0u - (a & 1)));
	}
	return r;
}
/* CRC of data followed by zeroPad zero bytes (crc_zeroPad: multiply the raw
 * state by x^(8*zeroPad) by square-and-multiply) */
uint32_t or_crc32(const uint8_t* data, size_t len, uint64_t zeroPad) {
	pthread_once(&or_crc_once, or_crc_build);
	uint32_t c = 0xFFFFFFFFu;
	for(size_t i = 0; i < len; i++) c = (c >> 8) ^ or_crc_tab[(c ^ data[i]) & 255];
	uint32_t xn = 0x00800000u; /* x^8 in reflected order */
	while(zeroPad) {
		if(zeroPad & 1) c = or_crc_mulmod(c, xn);
		xn = or_crc_mulmod(xn, xn);
		zeroPad >>= 1;
	}
	return ~c;
}

/* IFSC entries of one file (20 bytes per slice: MD5 then CRC32 little-endian,
 * last slice zero-padded to sliceSize) and the file MD5 (no padding). */
void or_hash_file(const uint8_t* data, size_t len, size_t sliceSize, uint8_t* ifsc, uint8_t fileMd5[16]) {
	size_t nslices = (len + sliceSize - 1) / sliceSize;
	for(size_t s = 0; s < nslices; s++) {
		size_t off = s * sliceSize;
		size_t n = len - off < sliceSize ? len - off : sliceSize;
		or_md5(data + off, n, sliceSize - n, ifsc + 20 * s);
		uint32_t crc = or_crc32(data + off, n, sliceSize - n);
		for(int b = 0; b < 4; b++) ifsc[20 * s + 16 + b] = (uint8_t)(crc >> (8 * b));
	}
	or_md5(data, len, 0, fileMd5);
}

uint32_t or_crc32_fast(const uint8_t* data, size_t len, uint64_t zeroPad);

/* ---------- seeded synthetic slices (the bytes of parpar_gb300/synth.py) ----------
 * Byte b of row `first + i` is byte b % 8 of splitmix64(seed*K1 + row*K2 + b/8);
 * filled over `threads` threads so the CPU arm can build multi-GiB inputs. */
typedef struct { uint8_t* dst; size_t pitch, bytes; unsigned n, nt, tid; uint64_t seed, first; } or_sjob;
static void* or_sworker(void* arg) {
	const or_sjob* j = (const or_sjob*)arg;
	for(unsigned i = j->tid; i < j->n; i += j->nt) {
		uint64_t base = j->seed * 0xD1342543DE82EF95ull + (j->first + i) * 0x9E3779B97F4A7C15ull;
		uint8_t* row = j->dst + (size_t)i * j->pitch;
		for(size_t u = 0; u * 8 < j->bytes; u++) {
			uint64_t z = base + u;
			z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
			z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
			z ^= z >> 31;
			size_t k = j->bytes - u * 8 < 8 ? j->bytes - u * 8 : 8;
			for(size_t b = 0; b < k; b++) row[u * 8 + b] = (uint8_t)(z >> (8 * b));
		}
	}
	return NULL;
}
void or_synth_fill(uint8_t* dst, size_t pitch, unsigned n, size_t bytes, uint64_t seed, uint64_t first, int threads) {
	if(threads < 1) threads = 1;
	if(threads > 256) threads = 256;
	pthread_t th[256];
	or_sjob jobs[256];
	for(int t = 0; t < threads; t++) {
		or_sjob jb = {dst, pitch, bytes, n, (unsigned)threads, (unsigned)t, seed, first};
		jobs[t] = jb;
	}
	for(int t = 0; t < threads; t++) pthread_create(&th[t], NULL, or_sworker, &jobs[t]);
	for(int t = 0; t < threads; t++) pthread_join(th[t], NULL);
}

/* ---------- MD5 of many equal-length buffers (threaded; hashing baseline) ---------- */
typedef struct { const uint8_t* base; size_t stride, len; const size_t* lens; uint64_t pad; unsigned n, nt, tid; uint8_t* md5; uint32_t* crc; } or_hjob;
static void* or_hworker(void* arg) {
	or_hjob* j = (or_hjob*)arg;
	for(unsigned i = j->tid; i < j->n; i += j->nt) {
		size_t l = j->lens ? j->lens[i] : j->len;
		uint64_t pad = j->lens ? (uint64_t)(j->len - l) : j->pad;
		or_md5(j->base + (size_t)i * j->stride, l, pad, j->md5 + 16 * (size_t)i);
		if(j->crc) j->crc[i] = or_crc32_fast(j->base + (size_t)i * j->stride, l, pad);
	}
	return NULL;
}
/* MD5 (+ optional CRC32) of n rows; row i holds lens[i] bytes zero-padded to len
 * (lens may be NULL: every row is `len` bytes). */
void or_hash_rows(const uint8_t* base, size_t stride, size_t len, const size_t* lens, unsigned n,
                  uint8_t* md5, uint32_t* crc, int threads) {
	pthread_once(&or_crc_once, or_crc_build);
	if(threads < 1) threads = 1;
	if(threads > 256) threads = 256;
	pthread_t th[256];
	or_hjob jobs[256];
	for(int t = 0; t < threads; t++) {
		or_hjob jb = {base, stride, len, lens, 0, n, (unsigned)threads, (unsigned)t, md5, crc};
		jobs[t] = jb;
	}
	for(int t = 0; t < threads; t++) pthread_create(&th[t], NULL, or_hworker, &jobs[t]);
	for(int t = 0; t < threads; t++) pthread_join(th[t], NULL);
}

/* ---------- CPU baseline: the reference's fastest method on this host ----------
 * or_recover_fast computes the same product as or_recover for zero-padded
 * input rows (lens = slice).  On aarch64 it restates the reference's NEON
 * split-nibble SHUFFLE method (gf16/gf16_shuffle_neon.c): per coefficient,
 * eight 16-byte tables (4 nibble positions x low/high result byte), 16 words
 * per step de-interleaved into low/high bytes with vld2q_u8, eight TBL
 * lookups per recovery row, accumulators for two recovery rows held in L1 and
 * re-interleaved with vst2q_u8.  Elsewhere it falls back to or_recover.
 * Used only as the timed CPU baseline; the tests check it against or_recover. */
#if defined(__aarch64__) && defined(__ARM_NEON)
#include <arm_neon.h>
#define OR_FAST_NEON 1
#define OR_CHUNK_WORDS 4096

typedef struct {
	const uint8_t* inputs; const uint16_t* coeffs; unsigned n, r; size_t slice; uint8_t* out;
	unsigned nthreads, tid;
} or_fjob;

static void or_nib_tables(uint16_t c, uint8x16_t tl[4], uint8x16_t th[4]) {
	uint8_t lo[4][16], hi[4][16];
	for(int q = 0; q < 4; q++)
		for(int v = 0; v < 16; v++) {
			uint16_t p = or_mul(c, (uint16_t)(v << (4 * q)));
			lo[q][v] = (uint8_t)p;
			hi[q][v] = (uint8_t)(p >> 8);
		}
	for(int q = 0; q < 4; q++) { tl[q] = vld1q_u8(lo[q]); th[q] = vld1q_u8(hi[q]); }
}

static void* or_fast_worker(void* arg) {
	or_fjob* j = (or_fjob*)arg;
	const size_t words = j->slice / 2;
	const size_t vecWords = words / 16 * 16;          /* NEON part; tail done with lookups */
	const unsigned nchunks = (unsigned)((vecWords + OR_CHUNK_WORDS - 1) / OR_CHUNK_WORDS);
	const unsigned pairs = (j->r + 1) / 2;
	uint8_t* acc = (uint8_t*)aligned_alloc(64, 4 * OR_CHUNK_WORDS); /* [row 0 lo|hi][row 1 lo|hi] */
	const size_t units = (size_t)nchunks * pairs;
	for(size_t u = j->tid; u < units; u += j->nthreads) {
		const unsigned ch = (unsigned)(u / pairs), pr = (unsigned)(u % pairs);
		const size_t w0 = (size_t)ch * OR_CHUNK_WORDS;
		const size_t nw = vecWords - w0 < OR_CHUNK_WORDS ? vecWords - w0 : OR_CHUNK_WORDS;
		const unsigned r0 = pr * 2, nr = (r0 + 1 < j->r) ? 2 : 1;
		memset(acc, 0, 4 * OR_CHUNK_WORDS);
		for(unsigned i = 0; i < j->n; i++) {
			uint8x16_t tl[2][4], th[2][4];
			for(unsigned o = 0; o < nr; o++) or_nib_tables(j->coeffs[(size_t)(r0 + o) * j->n + i], tl[o], th[o]);
			if(nr == 1) for(int q = 0; q < 4; q++) { tl[1][q] = vdupq_n_u8(0); th[1][q] = vdupq_n_u8(0); }
			const uint8_t* src = j->inputs + (size_t)i * j->slice + 2 * w0;
			const uint8x16_t m4 = vdupq_n_u8(15);
			for(size_t b = 0; b < nw / 16; b++) {
				uint8x16x2_t v = vld2q_u8(src + 32 * b);
				uint8x16_t n0 = vandq_u8(v.val[0], m4), n1 = vshrq_n_u8(v.val[0], 4);
				uint8x16_t n2 = vandq_u8(v.val[1], m4), n3 = vshrq_n_u8(v.val[1], 4);
				for(int o = 0; o < 2; o++) {
					uint8x16_t rl = veorq_u8(veorq_u8(vqtbl1q_u8(tl[o][0], n0), vqtbl1q_u8(tl[o][1], n1)),
					                         veorq_u8(vqtbl1q_u8(tl[o][2], n2), vqtbl1q_u8(tl[o][3], n3)));
					uint8x16_t rh = veorq_u8(veorq_u8(vqtbl1q_u8(th[o][0], n0), vqtbl1q_u8(th[o][1], n1)),
					                         veorq_u8(vqtbl1q_u8(th[o][2], n2), vqtbl1q_u8(th[o][3], n3)));
					uint8_t* al = acc + o * 2 * OR_CHUNK_WORDS + 16 * b;
					uint8_t* ah = al + OR_CHUNK_WORDS;
					vst1q_u8(al, veorq_u8(vld1q_u8(al), rl));
					vst1q_u8(ah, veorq_u8(vld1q_u8(ah), rh));
				}
			}
		}
		for(unsigned o = 0; o < nr; o++) {
			uint8_t* dst = j->out + (size_t)(r0 + o) * j->slice + 2 * w0;
			const uint8_t* al = acc + o * 2 * OR_CHUNK_WORDS;
			for(size_t b = 0; b < nw / 16; b++) {
				uint8x16x2_t z;
				z.val[0] = vld1q_u8(al + 16 * b);
				z.val[1] = vld1q_u8(al + OR_CHUNK_WORDS + 16 * b);
				vst2q_u8(dst + 32 * b, z);
			}
		}
	}
	free(acc);
	return NULL;
}
#endif

int or_recover_fast(const uint8_t* inputs, unsigned n, size_t slice, const uint16_t* coeffs, unsigned r,
                    uint8_t* out, int threads) {
	or_init();
	if(slice & 1) return -1;
	if(threads < 1) threads = 1;
	if(threads > 256) threads = 256;
#ifdef OR_FAST_NEON
	const size_t words = slice / 2, vecWords = words / 16 * 16;
	pthread_t th[256];
	or_fjob jobs[256];
	for(int t = 0; t < threads; t++) {
		or_fjob jb = {inputs, coeffs, n, r, slice, out, (unsigned)threads, (unsigned)t};
		jobs[t] = jb;
	}
	for(int t = 0; t < threads; t++) pthread_create(&th[t], NULL, or_fast_worker, &jobs[t]);
	for(int t = 0; t < threads; t++) pthread_join(th[t], NULL);
	if(vecWords < words) { /* tail words with the table method */
		for(unsigned row = 0; row < r; row++) {
			uint8_t* dst = out + (size_t)row * slice + 2 * vecWords;
			memset(dst, 0, 2 * (words - vecWords));
			for(unsigned i = 0; i < n; i++)
				or_muladd_region(dst, inputs + (size_t)i * slice + 2 * vecWords, words - vecWords, coeffs[(size_t)row * n + i]);
		}
	}
	return 0;
#else
	size_t* lens = (size_t*)malloc(sizeof(size_t) * (n ? n : 1));
	if(!lens) return -2;
	for(unsigned i = 0; i < n; i++) lens[i] = slice;
	int rc = or_recover_coeffs(inputs, lens, coeffs, n, slice, r, out, threads);
	free(lens);
	return rc;
#endif
}

const char* or_fast_method(void) {
#ifdef OR_FAST_NEON
	return "NEON split-nibble shuffle (restating the reference's SHUFFLE_NEON method)";
#else
	return "portable LOOKUP (the reference's portable method)";
#endif
}

/* CRC32 for the baseline's hashing: the ARMv8 CRC32 instructions where the
 * host has them (the reference's ARMCRC hasher), else the table method. */
#if defined(__aarch64__) && defined(__ARM_FEATURE_CRC32)
#include <arm_acle.h>
uint32_t or_crc32_fast(const uint8_t* data, size_t len, uint64_t zeroPad) {
	uint32_t c = 0xFFFFFFFFu;
	size_t i = 0;
	for(; i + 8 <= len; i += 8) { uint64_t v; memcpy(&v, data + i, 8); c = __crc32d(c, v); }
	for(; i < len; i++) c = __crc32b(c, data[i]);
	/* zero padding by x^(8n) as in or_crc32 */
	uint32_t xn = 0x00800000u;
	while(zeroPad) {
		if(zeroPad & 1) c = or_crc_mulmod(c, xn);
		xn = or_crc_mulmod(xn, xn);
		zeroPad >>= 1;
	}
	return ~c;
}
#else
uint32_t or_crc32_fast(const uint8_t* data, size_t len, uint64_t zeroPad) { return or_crc32(data, len, zeroPad); }
#endif

/* ---------- CPU baseline: carry-less multiply method (SVE2) ----------
 * Restates the reference's CLMUL_SVE2 method (gf16/gf16_clmul_sve2.c), its
 * automatic choice on SVE2 hosts such as Grace: each 16-bit word a = a1 x^8 + a0
 * times c = c1 x^8 + c0 as three 8x8 carry-less products (Karatsuba: a0c0,
 * a1c1, (a0+a1)(c0+c1)) with PMULLB/PMULLT on the de-interleaved low/high
 * bytes (even and odd words), accumulated unreduced over the inputs (the
 * reduction is linear, so it is done once per output word at the end):
 *     product = HH x^16 + (MM + LL + HH) x^8 + LL,   lo16 + hi16 x^16
 *     result  = lo16 ^ red[hi16],   red[h] = h * x^16 mod 0x1100B (h < 2^15)
 * Four inputs per pass into one output with the six accumulators (LL, MM, HH
 * x even/odd) in registers, combined with three-input XORs.  Compiled only
 * when the compiler accepts SVE2 (OR_ENABLE_SVE2, tried by the loader) and
 * used only when the CPU reports SVE2. */
#if defined(__aarch64__) && defined(OR_ENABLE_SVE2)
#include <sys/auxv.h>
#ifndef HWCAP2_SVE2
#define HWCAP2_SVE2 (1 << 1)
#endif
#pragma GCC push_options
#pragma GCC target("+sve2")
#include <arm_sve.h>

#define OR_CL_CHUNK 2048   /* words per unit: 4 inputs x 4 KiB + 12 KiB of accumulators in L1 */

static uint16_t or_red_tab[32768];
static pthread_once_t or_red_once = PTHREAD_ONCE_INIT;
static void or_red_build(void) {
	for(uint32_t h = 0; h < 32768; h++) or_red_tab[h] = or_mul((uint16_t)h, 0x100B);
}

typedef struct {
	const uint8_t* inputs; const uint16_t* coeffs; unsigned n, r; size_t slice; uint8_t* out;
	unsigned nthreads, tid;
} or_cljob;

static void* or_clmul_worker(void* arg) {
	or_cljob* j = (or_cljob*)arg;
	const size_t VLW = svcntb();                       /* words per svld2 block */
	const size_t words = j->slice / 2;
	const size_t vecWords = words / OR_CL_CHUNK * OR_CL_CHUNK;
	const size_t nchunks = vecWords / OR_CL_CHUNK;
	const size_t blocks = OR_CL_CHUNK / VLW;
	uint8_t* accb = (uint8_t*)aligned_alloc(64, 6 * blocks * svcntb());
	const svbool_t pt = svptrue_b8();
	const size_t units = nchunks * j->r;
	for(size_t u = j->tid; u < units; u += j->nthreads) {
		const size_t ch = u / j->r;
		const unsigned row = (unsigned)(u % j->r);
		const size_t w0 = ch * OR_CL_CHUNK;
		memset(accb, 0, 6 * blocks * svcntb());
		for(unsigned i = 0; i < j->n; i += 4) {
			const unsigned k = j->n - i < 4 ? j->n - i : 4;
			const uint8_t* src[4];
			uint16_t cv[4];
			for(unsigned t = 0; t < 4; t++) {
				cv[t] = t < k ? j->coeffs[(size_t)row * j->n + i + t] : 0;   /* zero: adds nothing */
				src[t] = j->inputs + (size_t)(i + (t < k ? t : 0)) * j->slice + 2 * w0;
			}
			/* coefficient byte vectors (SVE types cannot form arrays) */
			const svuint8_t a_c0 = svdup_n_u8((uint8_t)cv[0]), a_c1 = svdup_n_u8((uint8_t)(cv[0] >> 8)),
			                a_cm = svdup_n_u8((uint8_t)(cv[0] ^ (cv[0] >> 8)));
			const svuint8_t b_c0 = svdup_n_u8((uint8_t)cv[1]), b_c1 = svdup_n_u8((uint8_t)(cv[1] >> 8)),
			                b_cm = svdup_n_u8((uint8_t)(cv[1] ^ (cv[1] >> 8)));
			const svuint8_t c_c0 = svdup_n_u8((uint8_t)cv[2]), c_c1 = svdup_n_u8((uint8_t)(cv[2] >> 8)),
			                c_cm = svdup_n_u8((uint8_t)(cv[2] ^ (cv[2] >> 8)));
			const svuint8_t d_c0 = svdup_n_u8((uint8_t)cv[3]), d_c1 = svdup_n_u8((uint8_t)(cv[3] >> 8)),
			                d_cm = svdup_n_u8((uint8_t)(cv[3] ^ (cv[3] >> 8)));
			for(size_t b = 0; b < blocks; b++) {
				uint8_t* ab = accb + 6 * b * svcntb();
				svuint16_t lle = svld1_u16(pt, (const uint16_t*)(ab + 0 * svcntb()));
				svuint16_t llo = svld1_u16(pt, (const uint16_t*)(ab + 1 * svcntb()));
				svuint16_t mme = svld1_u16(pt, (const uint16_t*)(ab + 2 * svcntb()));
				svuint16_t mmo = svld1_u16(pt, (const uint16_t*)(ab + 3 * svcntb()));
				svuint16_t hhe = svld1_u16(pt, (const uint16_t*)(ab + 4 * svcntb()));
				svuint16_t hho = svld1_u16(pt, (const uint16_t*)(ab + 5 * svcntb()));
				/* inputs a, b, then c, d: two products per three-input XOR */
#define OR_CL_PAIR(P, Q, SP, SQ) do { \
					svuint8x2_t dp = svld2_u8(pt, (SP) + 2 * b * VLW); \
					svuint8x2_t dq = svld2_u8(pt, (SQ) + 2 * b * VLW); \
					svuint8_t p0 = svget2_u8(dp, 0), p1 = svget2_u8(dp, 1), pm = sveor_u8_x(pt, p0, p1); \
					svuint8_t q0 = svget2_u8(dq, 0), q1 = svget2_u8(dq, 1), qm = sveor_u8_x(pt, q0, q1); \
					lle = sveor3_u16(lle, svpmullb_u16(p0, P##_c0), svpmullb_u16(q0, Q##_c0)); \
					llo = sveor3_u16(llo, svpmullt_u16(p0, P##_c0), svpmullt_u16(q0, Q##_c0)); \
					hhe = sveor3_u16(hhe, svpmullb_u16(p1, P##_c1), svpmullb_u16(q1, Q##_c1)); \
					hho = sveor3_u16(hho, svpmullt_u16(p1, P##_c1), svpmullt_u16(q1, Q##_c1)); \
					mme = sveor3_u16(mme, svpmullb_u16(pm, P##_cm), svpmullb_u16(qm, Q##_cm)); \
					mmo = sveor3_u16(mmo, svpmullt_u16(pm, P##_cm), svpmullt_u16(qm, Q##_cm)); \
				} while(0)
				OR_CL_PAIR(a, b, src[0], src[1]);
				OR_CL_PAIR(c, d, src[2], src[3]);
#undef OR_CL_PAIR
				svst1_u16(pt, (uint16_t*)(ab + 0 * svcntb()), lle);
				svst1_u16(pt, (uint16_t*)(ab + 1 * svcntb()), llo);
				svst1_u16(pt, (uint16_t*)(ab + 2 * svcntb()), mme);
				svst1_u16(pt, (uint16_t*)(ab + 3 * svcntb()), mmo);
				svst1_u16(pt, (uint16_t*)(ab + 4 * svcntb()), hhe);
				svst1_u16(pt, (uint16_t*)(ab + 5 * svcntb()), hho);
			}
		}
		/* one reduction per output word */
		uint8_t* dst = j->out + (size_t)row * j->slice + 2 * w0;
		const size_t half = VLW / 2;                    /* 16-bit lanes per vector */
		for(size_t b = 0; b < blocks; b++) {
			const uint16_t* a = (const uint16_t*)(accb + 6 * b * svcntb());
			for(size_t q = 0; q < half; q++)
				for(unsigned odd = 0; odd < 2; odd++) {
					const uint16_t ll = a[(0 + odd) * half + q], mm = a[(2 + odd) * half + q], hh = a[(4 + odd) * half + q];
					const uint16_t mid = (uint16_t)(mm ^ ll ^ hh);
					const uint16_t lo = (uint16_t)(ll ^ (uint16_t)(mid << 8));
					const uint16_t hi = (uint16_t)(hh ^ (mid >> 8));
					const uint16_t v = (uint16_t)(lo ^ or_red_tab[hi & 32767]);
					const size_t w = b * VLW + 2 * q + odd;
					dst[2 * w] = (uint8_t)v;
					dst[2 * w + 1] = (uint8_t)(v >> 8);
				}
		}
	}
	free(accb);
	return NULL;
}
#pragma GCC pop_options

static int or_have_sve2(void) { return (getauxval(AT_HWCAP2) & HWCAP2_SVE2) != 0; }
#endif

#if defined(__aarch64__)
/* The same method with NEON polynomial multiplies (the reference's
 * CLMUL_NEON, gf16/gf16_clmul_neon.c, its automatic choice on NEON hosts
 * without SVE2): vmull_p8 / vmull_high_p8 on the low and high eight words of
 * the de-interleaved bytes, six products per input and 16 words, accumulated
 * unreduced over four inputs per pass, one table reduction per output word. */
#include <arm_neon.h>
#ifndef OR_CL_CHUNK
#define OR_CL_CHUNK 2048
#endif
static uint16_t or_nred_tab[32768];
static pthread_once_t or_nred_once = PTHREAD_ONCE_INIT;
static void or_nred_build(void) {
	for(uint32_t h = 0; h < 32768; h++) or_nred_tab[h] = or_mul((uint16_t)h, 0x100B);
}
typedef struct {
	const uint8_t* inputs; const uint16_t* coeffs; unsigned n, r; size_t slice; uint8_t* out;
	unsigned nthreads, tid;
} or_ncljob;

static void* or_nclmul_worker(void* arg) {
	or_ncljob* j = (or_ncljob*)arg;
	const size_t words = j->slice / 2;
	const size_t nchunks = words / OR_CL_CHUNK;
	const size_t blocks = OR_CL_CHUNK / 16;
	uint16_t* acc = (uint16_t*)aligned_alloc(64, blocks * 6 * 16 * sizeof(uint16_t)); /* per block: LL, MM, HH x 16 words */
	const size_t units = nchunks * j->r;
	for(size_t u = j->tid; u < units; u += j->nthreads) {
		const size_t ch = u / j->r;
		const unsigned row = (unsigned)(u % j->r);
		const size_t w0 = ch * OR_CL_CHUNK;
		memset(acc, 0, blocks * 6 * 16 * sizeof(uint16_t));
		for(unsigned i = 0; i < j->n; i += 4) {
			const unsigned k = j->n - i < 4 ? j->n - i : 4;
			const uint8_t* src[4];
			poly8x16_t c0[4], c1[4], cm[4];
			for(unsigned t = 0; t < 4; t++) {
				const uint16_t c = t < k ? j->coeffs[(size_t)row * j->n + i + t] : 0;   /* zero: adds nothing */
				src[t] = j->inputs + (size_t)(i + (t < k ? t : 0)) * j->slice + 2 * w0;
				c0[t] = vreinterpretq_p8_u8(vdupq_n_u8((uint8_t)c));
				c1[t] = vreinterpretq_p8_u8(vdupq_n_u8((uint8_t)(c >> 8)));
				cm[t] = vreinterpretq_p8_u8(vdupq_n_u8((uint8_t)(c ^ (c >> 8))));
			}
			for(size_t b = 0; b < blocks; b++) {
				uint16_t* ab = acc + b * 96;
				uint16x8_t ll0 = vld1q_u16(ab), ll1 = vld1q_u16(ab + 8);
				uint16x8_t mm0 = vld1q_u16(ab + 16), mm1 = vld1q_u16(ab + 24);
				uint16x8_t hh0 = vld1q_u16(ab + 32), hh1 = vld1q_u16(ab + 40);
				for(unsigned t = 0; t < 4; t++) {
					const uint8x16x2_t d = vld2q_u8(src[t] + 32 * b);
					const poly8x16_t a0 = vreinterpretq_p8_u8(d.val[0]), a1 = vreinterpretq_p8_u8(d.val[1]);
					const poly8x16_t am = vreinterpretq_p8_u8(veorq_u8(d.val[0], d.val[1]));
					ll0 = veorq_u16(ll0, vreinterpretq_u16_p16(vmull_p8(vget_low_p8(a0), vget_low_p8(c0[t]))));
					ll1 = veorq_u16(ll1, vreinterpretq_u16_p16(vmull_high_p8(a0, c0[t])));
					hh0 = veorq_u16(hh0, vreinterpretq_u16_p16(vmull_p8(vget_low_p8(a1), vget_low_p8(c1[t]))));
					hh1 = veorq_u16(hh1, vreinterpretq_u16_p16(vmull_high_p8(a1, c1[t])));
					mm0 = veorq_u16(mm0, vreinterpretq_u16_p16(vmull_p8(vget_low_p8(am), vget_low_p8(cm[t]))));
					mm1 = veorq_u16(mm1, vreinterpretq_u16_p16(vmull_high_p8(am, cm[t])));
				}
				vst1q_u16(ab, ll0); vst1q_u16(ab + 8, ll1);
				vst1q_u16(ab + 16, mm0); vst1q_u16(ab + 24, mm1);
				vst1q_u16(ab + 32, hh0); vst1q_u16(ab + 40, hh1);
			}
		}
		uint8_t* dst = j->out + (size_t)row * j->slice + 2 * w0;
		for(size_t b = 0; b < blocks; b++) {
			const uint16_t* a = acc + b * 96;
			for(unsigned q = 0; q < 16; q++) {
				const uint16_t ll = a[q], mm = a[16 + q], hh = a[32 + q];
				const uint16_t mid = (uint16_t)(mm ^ ll ^ hh);
				const uint16_t lo = (uint16_t)(ll ^ (uint16_t)(mid << 8));
				const uint16_t hi = (uint16_t)(hh ^ (mid >> 8));
				const uint16_t v = (uint16_t)(lo ^ or_nred_tab[hi & 32767]);
				const size_t w = b * 16 + q;
				dst[2 * w] = (uint8_t)v;
				dst[2 * w + 1] = (uint8_t)(v >> 8);
			}
		}
	}
	free(acc);
	return NULL;
}
#endif

/* Which carry-less multiply form or_recover_clmul uses on this host. */
const char* or_clmul_method(void) {
#if defined(__aarch64__) && defined(OR_ENABLE_SVE2)
	if(or_have_sve2()) return "SVE2 carry-less multiply (restating the reference's CLMUL_SVE2 method, its automatic choice on SVE2 hosts)";
#endif
#if defined(__aarch64__)
	return "NEON carry-less multiply (restating the reference's CLMUL_NEON method, its automatic choice on NEON hosts without SVE2)";
#else
	return "";
#endif
}

/* The carry-less multiply method over zero-padded rows (SVE2 where the CPU
 * has it, else NEON); returns -3 where it is not available (not aarch64). */
int or_recover_clmul(const uint8_t* inputs, unsigned n, size_t slice, const uint16_t* coeffs, unsigned r,
                     uint8_t* out, int threads) {
#if defined(__aarch64__)
	or_init();
	if(slice & 1) return -1;
	if(threads < 1) threads = 1;
	if(threads > 256) threads = 256;
#if defined(OR_ENABLE_SVE2)
	const int sve2 = or_have_sve2();
#else
	const int sve2 = 0;
#endif
	if(!sve2) {
		pthread_once(&or_nred_once, or_nred_build);
		const size_t words = slice / 2, vecWords = words / OR_CL_CHUNK * OR_CL_CHUNK;
		pthread_t th[256];
		or_ncljob jobs[256];
		for(int t = 0; t < threads; t++) {
			or_ncljob jb = {inputs, coeffs, n, r, slice, out, (unsigned)threads, (unsigned)t};
			jobs[t] = jb;
		}
		for(int t = 0; t < threads; t++) pthread_create(&th[t], NULL, or_nclmul_worker, &jobs[t]);
		for(int t = 0; t < threads; t++) pthread_join(th[t], NULL);
		if(vecWords < words)
			for(unsigned row = 0; row < r; row++) {
				uint8_t* dst = out + (size_t)row * slice + 2 * vecWords;
				memset(dst, 0, 2 * (words - vecWords));
				for(unsigned i = 0; i < n; i++)
					or_muladd_region(dst, inputs + (size_t)i * slice + 2 * vecWords, words - vecWords, coeffs[(size_t)row * n + i]);
			}
		return 0;
	}
#endif
#if defined(__aarch64__) && defined(OR_ENABLE_SVE2)
	pthread_once(&or_red_once, or_red_build);
	const size_t words = slice / 2, vecWords = words / OR_CL_CHUNK * OR_CL_CHUNK;
	pthread_t th[256];
	or_cljob jobs[256];
	for(int t = 0; t < threads; t++) {
		or_cljob jb = {inputs, coeffs, n, r, slice, out, (unsigned)threads, (unsigned)t};
		jobs[t] = jb;
	}
	for(int t = 0; t < threads; t++) pthread_create(&th[t], NULL, or_clmul_worker, &jobs[t]);
	for(int t = 0; t < threads; t++) pthread_join(th[t], NULL);
	if(vecWords < words) { /* tail words with the table method */
		for(unsigned row = 0; row < r; row++) {
			uint8_t* dst = out + (size_t)row * slice + 2 * vecWords;
			memset(dst, 0, 2 * (words - vecWords));
			for(unsigned i = 0; i < n; i++)
				or_muladd_region(dst, inputs + (size_t)i * slice + 2 * vecWords, words - vecWords, coeffs[(size_t)row * n + i]);
		}
	}
	return 0;
#else
	(void)inputs; (void)n; (void)slice; (void)coeffs; (void)r; (void)out; (void)threads;
	return -3;
#endif
}
