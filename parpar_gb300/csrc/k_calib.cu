// Calibration: the device's measured three-input LOP3 throughput, the
// denominator of the integer-ALU roofline of the multiply-accumulate kernels
// (a GF(2^16) multiply-accumulate of one 16-bit word costs 2 LOP3 in the
// 32-way bit-sliced form).  The kernel runs eight interleaved XOR3 chains per
// thread at full occupancy; each step reads two other chains so no chain can
// be simplified away, and the final value is kept live by a data-dependent
// store that never happens for these seeds.
#include "common.cuh"
#include "kernels.h"

namespace p2c {

constexpr int CALIB_THREADS = 512;
constexpr int CALIB_UNROLL = 8;   // x 8 chains = 64 LOP3 per loop trip

__global__ void __launch_bounds__(CALIB_THREADS) k_lop3_rate(uint32_t* sink, int iters) {
	uint32_t a[8];
#pragma unroll
	for(int j = 0; j < 8; j++) a[j] = threadIdx.x * (2u * j + 1u) + blockIdx.x * 0x9E3779B9u + j;
	for(int it = 0; it < iters; it++) {
#pragma unroll
		for(int u = 0; u < CALIB_UNROLL; u++)
#pragma unroll
			for(int j = 0; j < 8; j++)
				asm volatile("lop3.b32 %0, %0, %1, %2, 0x96;" : "+r"(a[j]) : "r"(a[(j + 1) & 7]), "r"(a[(j + 5) & 7]));
	}
	uint32_t v = 0;
#pragma unroll
	for(int j = 0; j < 8; j++) v ^= a[j];
	if(v == 0x5EEDF00Du && iters < 0) sink[blockIdx.x] = v;
}

int lop3_rate(double* opsPerSec, cudaStream_t st) {
	int dev = 0, sms = 0;
	P2C_CUDA_TRY(cudaGetDevice(&dev));
	P2C_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
	int occ = 1;
	P2C_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_lop3_rate, CALIB_THREADS, 0));
	const unsigned grid = (unsigned)sms * (unsigned)std::max(occ, 1);
	const int iters = 4000;
	cudaEvent_t e0, e1;
	P2C_CUDA_TRY(cudaEventCreate(&e0));
	P2C_CUDA_TRY(cudaEventCreate(&e1));
	k_lop3_rate<<<grid, CALIB_THREADS, 0, st>>>(nullptr, iters); // warm-up
	float best = 0.f;
	for(int rep = 0; rep < 3; rep++) {
		cudaEventRecord(e0, st);
		k_lop3_rate<<<grid, CALIB_THREADS, 0, st>>>(nullptr, iters * 5);
		cudaEventRecord(e1, st);
		cudaError_t e = cudaEventSynchronize(e1);
		if(e != cudaSuccess) {
			cudaEventDestroy(e0); cudaEventDestroy(e1);
			set_error("lop3 calibration: %s", cudaGetErrorString(e));
			return -1;
		}
		float ms = 0.f;
		cudaEventElapsedTime(&ms, e0, e1);
		if(rep == 0 || ms < best) best = ms;
	}
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	P2C_CUDA_TRY(cudaGetLastError());
	const double ops = (double)grid * CALIB_THREADS * (double)iters * 5 * CALIB_UNROLL * 8;
	*opsPerSec = best > 0.f ? ops / (best * 1e-3) : 0.0;
	return 0;
}

} // namespace p2c
