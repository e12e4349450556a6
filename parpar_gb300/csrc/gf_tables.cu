// Per-device GF(2^16) tables (antilog, log, PAR2 input logs) and the
// thread-local error string behind par2cuda_last_error().
#include "common.cuh"
#include "kernels.h"

#include <cstdarg>
#include <cstdio>
#include <mutex>
#include <vector>

namespace p2c {

static thread_local char g_err[512];
void set_error(const char* fmt, ...) {
	va_list ap;
	va_start(ap, fmt);
	vsnprintf(g_err, sizeof(g_err), fmt, ap);
	va_end(ap);
}
const char* get_error() { return g_err; }

// Host construction follows the field definition: 2 is a generator of
// GF(2^16) mod 0x1100B; PAR2 input i uses the i-th exponent (from 1) coprime
// with 65535 (not divisible by 3, 5, 17 or 257) — gf16/gfmat_coeff.c:6-34.
static void host_tables(std::vector<uint16_t>& exp, std::vector<uint16_t>& log, std::vector<uint16_t>& inLog) {
	exp.assign(131072, 0);
	log.assign(65536, 0);
	inLog.assign(32768, 0);
	uint32_t n = 1;
	for(uint32_t e = 0; e < 65535; e++) {
		exp[e] = exp[e + 65535] = (uint16_t)n;
		log[n] = (uint16_t)e;
		n <<= 1;
		if(n & 0x10000) n ^= P2C_POLY;
	}
	exp[131070] = exp[0];
	exp[131071] = exp[1];
	uint32_t e = 0;
	for(int i = 0; i < 32768; i++) {
		do { e++; } while(e % 3 == 0 || e % 5 == 0 || e % 17 == 0 || e % 257 == 0);
		inLog[i] = (uint16_t)e;
	}
}

static std::mutex g_tab_mutex;
static GfTables g_tabs[64];
static bool g_tab_ready[64];

int gf_tables(int device, GfTables* out) {
	if(device < 0 || device >= 64) { set_error("device %d out of range", device); return -1; }
	std::lock_guard<std::mutex> lk(g_tab_mutex);
	if(!g_tab_ready[device]) {
		std::vector<uint16_t> e, l, il;
		host_tables(e, l, il);
		int prev = 0;
		P2C_CUDA_TRY(cudaGetDevice(&prev));
		P2C_CUDA_TRY(cudaSetDevice(device));
		uint16_t* d = nullptr;
		P2C_CUDA_TRY(cudaMalloc(&d, (131072 + 65536 + 32768) * sizeof(uint16_t)));
		P2C_CUDA_TRY(cudaMemcpy(d, e.data(), 131072 * 2, cudaMemcpyHostToDevice));
		P2C_CUDA_TRY(cudaMemcpy(d + 131072, l.data(), 65536 * 2, cudaMemcpyHostToDevice));
		P2C_CUDA_TRY(cudaMemcpy(d + 131072 + 65536, il.data(), 32768 * 2, cudaMemcpyHostToDevice));
		P2C_CUDA_TRY(cudaSetDevice(prev));
		g_tabs[device].exp = d;
		g_tabs[device].log = d + 131072;
		g_tabs[device].inLog = d + 131072 + 65536;
		g_tab_ready[device] = true;
	}
	*out = g_tabs[device];
	return 0;
}

// host copy of the input-log table (for the engine's set_coeffs)
const uint16_t* host_input_logs() {
	static std::vector<uint16_t> il;
	static std::once_flag once;
	std::call_once(once, [] { std::vector<uint16_t> e, l; host_tables(e, l, il); });
	return il.data();
}

} // namespace p2c
