// par2cuda_muladd_noalloc: the comb multiply-accumulate with its scratch in a
// fixed, library-owned device array instead of caller-provided or allocated
// memory.
//
// Why: par2cuda_muladd needs a scratch buffer for the per-call index bytes
// (the coefficient bits regrouped for the XOR-combination tables).  Some
// callers cannot provide or allocate one: an application that hands the
// library only its input and output buffers under a fixed device-memory
// budget, or a latency-sensitive submission loop that must not call
// cudaMalloc (which may synchronise the device and stall work already queued
// on other streams).  This entry point needs neither.
//
// Limit: the scratch is P2C_NOALLOC_SCRATCH_BYTES (4 MiB), enough for
// num_rec * ceil(num_in / 8) <= 262144 (e.g. 4096 recovery slices x 512
// inputs, or 200 x 10480).  Every device that loads the library holds these
// 4 MiB until the process exits.
//
// Sharing: all calls on a device use the same array and it keeps the last
// call's contents.  Each call rewrites the index bytes it reads before
// reading them, so nothing has to start at zero; but two calls whose work
// overlaps on the GPU (different streams, no ordering between them) race on
// the array and give wrong results — order such calls on one stream or with
// events.
//
// Set-up: the first call on a device (with that device current) looks up the
// array's device address with cudaGetSymbolAddress and caches it; make that
// first call before any stream capture on the device.  The cached address is
// valid for the life of the device's primary context: a caller that resets
// the device (cudaDeviceReset) must not use this entry point afterwards, as
// the module reloads and the array can move.  The call performs no
// allocation of any kind.
#include "common.cuh"
#include "kernels.h"

#include <mutex>

#define P2C_NOALLOC_SCRATCH_BYTES (4u << 20)
#define P2C_NOALLOC_MAX_DEVICES 64

// file-scope device scratch; device code could name it directly, host code
// only uses the address obtained below
static __device__ __align__(256) uint8_t g_noalloc_scratch[P2C_NOALLOC_SCRATCH_BYTES];

static std::mutex g_noalloc_mutex;
static void* g_noalloc_ptr[P2C_NOALLOC_MAX_DEVICES];

// address of this device's scratch array (looked up once per device, with the
// device current)
static int noalloc_scratch(void** out) {
	int dev = 0;
	P2C_CUDA_TRY(cudaGetDevice(&dev));
	if(dev < 0 || dev >= P2C_NOALLOC_MAX_DEVICES) { p2c::set_error("device %d out of range", dev); return -1; }
	std::lock_guard<std::mutex> lk(g_noalloc_mutex);
	if(!g_noalloc_ptr[dev]) {
		void* p = nullptr;
		cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
		if(e != cudaSuccess || !p) {
			p2c::set_error("cudaGetSymbolAddress(scratch) failed on device %d: %s", dev, cudaGetErrorString(e));
			return -1;
		}
		g_noalloc_ptr[dev] = p;
	}
	*out = g_noalloc_ptr[dev];
	return 0;
}

extern "C" int par2cuda_muladd_noalloc(const uint16_t* d_in, size_t in_pitch_words, unsigned num_in,
                                       const uint16_t* d_coeff, uint16_t* d_rec, size_t rec_pitch_words,
                                       unsigned num_rec, size_t n_words, int accumulate, void* stream) {
	if((in_pitch_words & 1) || (rec_pitch_words & 1)) { p2c::set_error("row pitches must be even (whole u32 pairs)"); return -1; }
	const size_t need = p2c::idx_bytes(num_rec, num_in);
	if(need > P2C_NOALLOC_SCRATCH_BYTES) {
		p2c::set_error("par2cuda_muladd_noalloc: %u recovery x %u inputs need %zu bytes of scratch, the built-in limit is %u "
		               "(num_rec * ceil(num_in/8) <= %u); split the inputs over several calls with accumulate = 1",
		               num_rec, num_in, need, P2C_NOALLOC_SCRATCH_BYTES, P2C_NOALLOC_SCRATCH_BYTES / 16);
		return -1;
	}
	void* scratch = nullptr;
	if(noalloc_scratch(&scratch)) return -1;
	cudaStream_t st = (cudaStream_t)stream;
	uint4* idx = reinterpret_cast<uint4*>(scratch);
	if(p2c::coeff_to_idx(d_coeff, num_rec, num_in, idx, st)) return -1;
	return p2c::comb_muladd(d_in, in_pitch_words, num_in, idx, d_rec, rec_pitch_words, num_rec, n_words, accumulate, 0, st);
}
