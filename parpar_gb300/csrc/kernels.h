// Host-side launchers of the device kernels (all asynchronous on `st`).
#pragma once
#include "common.cuh"

namespace p2c {

// device GF tables for `device` (built on first use, kept until exit)
int gf_tables(int device, GfTables* out);

// zero the bytes of each row at and past lens[row] (or sliceBytes when dLens is
// null), compute the internal checksum over roundup(sliceBytes, 8) bytes and
// either store it in the row's checksum block (verify = 0) or compare it with
// the carried block into dFlags[row] (verify = 1).  dCkAcc: nRows x u64 scratch.
int rows_cksum(uint16_t* rows, size_t pitchWords, unsigned nRows, const uint32_t* dLens, size_t sliceBytes,
               unsigned long long* dCkAcc, int verify, uint8_t* dFlags, const GfTables& gt, cudaStream_t st);

// index bytes for the comb kernel from PAR2 logs (dInLogs[nIn]) and recovery
// exponents (dOutExp[R]) or from an explicit coefficient matrix
// dCustom[nIn][R]; optionally also writes the coefficients [R][nIn]
int make_idx(const uint16_t* dInLogs, const uint16_t* dCustom, const uint16_t* dOutExp, unsigned R, unsigned nIn,
             uint4* dIdx, uint16_t* dCoeffOut, const GfTables& gt, cudaStream_t st);
// index bytes from a coefficient matrix dCoeff[R][nIn]
int coeff_to_idx(const uint16_t* dCoeff, unsigned R, unsigned nIn, uint4* dIdx, cudaStream_t st);
// index bytes of PAR2 coefficients from input numbers dNums[nIn] and exponents dExp[R]
int par2_idx(const uint16_t* dNums, const uint16_t* dExp, unsigned R, unsigned nIn, uint4* dIdx, const GfTables& gt,
             cudaStream_t st);
int par2_coeffs(const uint16_t* dNums, const uint16_t* dExp, unsigned R, unsigned nIn, uint16_t* dCoeff,
                const GfTables& gt, cudaStream_t st);
inline size_t idx_bytes(unsigned R, unsigned nIn) { return (size_t)R * ((nIn + 7) / 8) * 16; }

// rec[r][0..nWords) (^)= sum_i c(r,i) in[i][0..nWords), the comb kernel
int comb_muladd(const uint16_t* in, size_t inPitch, unsigned nIn, const uint4* idx, uint16_t* rec, size_t recPitch,
                unsigned R, size_t nWords, int accumulate, int shape, cudaStream_t st);

// one job of a batched multiply-accumulate (device-resident descriptor;
// same layout as par2cuda_batch_job in include/par2cuda.h)
struct BatchJob {
	const uint16_t* in; size_t inPitch; unsigned nIn;
	const uint4* idx;              // index bytes (k_coeff_to_idx layout)
	uint16_t* rec; size_t recPitch; unsigned R;
	int accumulate;
	unsigned long long unitBase;   // first work unit of this job (ascending)
};
unsigned long long comb_units(unsigned R, size_t nWords, int shape);
int comb_batched(const BatchJob* dJobs, unsigned nJobs, unsigned long long totalUnits, unsigned long long* dCounter,
                 int shape, cudaStream_t st);

// process-wide CTA shape override for the comb kernel (0 = choose from R); returns the previous value
int set_comb_shape(int shape);
// shape chosen for R when none is set
int comb_auto_shape(unsigned R);
int comb_shape_for(unsigned R);  // the shape the next comb call with R rows uses
// reads and clears the device error flag of the comb kernels (1 = a bounded wait timed out)
int comb_error_take();
// measured three-input LOP3 throughput of the current device (ops/s)
int lop3_rate(double* opsPerSec, cudaStream_t st);
// one MD5 stream on one thread, data in registers: bytes/s
int md5_chain_rate(double* bytesPerSec, cudaStream_t st);

// bit-sliced LOP3 kernel and split-nibble table kernel (same contract, coefficient matrix [R][nIn])
int xor_planes_muladd(const uint16_t* in, size_t inPitch, unsigned nIn, const uint16_t* coeff, uint16_t* rec,
                      size_t recPitch, unsigned R, size_t nWords, int accumulate, cudaStream_t st);
int nibble_muladd_t(const uint16_t* in, size_t inPitch, unsigned nIn, const uint16_t* coeff, uint16_t* rec,
                    size_t recPitch, unsigned R, size_t nWords, int accumulate, const GfTables& gt, cudaStream_t st);

// per-row MD5+CRC32 of rows zero-padded to sliceBytes (20-byte IFSC entries)
int slice_hash(const void* rows, size_t pitchBytes, unsigned n, const uint32_t* dLens, size_t sliceBytes,
               uint8_t* dOut, cudaStream_t st);
// per-file MD5; file f spans consecutive rows from dFirstRow[f], dFileLen[f] bytes
int file_md5(const void* rows, size_t pitchBytes, unsigned nFiles, const uint64_t* dFileLen, const uint32_t* dFirstRow,
             size_t sliceBytes, uint8_t* dOut, cudaStream_t st, unsigned filesPerBlock = 1);
// MD5 of (prefix[i] ++ row i's first dataLen bytes)
int rows_md5(const void* rows, size_t pitchBytes, unsigned n, size_t dataLen, const uint8_t* dPrefix, unsigned prefixLen,
             uint8_t* dOut, cudaStream_t st);

// tensor-core (tcgen05, e4m3 0/1 operands, fp32 accumulators) variant, coefficient matrix [R][nIn]
int tc_muladd(const uint16_t* in, size_t inPitch, unsigned nIn, const uint16_t* coeff, uint16_t* rec, size_t recPitch,
              unsigned R, size_t nWords, int accumulate, bool fp8, void* scratch, size_t scratchBytes, cudaStream_t st);
size_t tc_scratch_bytes(unsigned R, unsigned nIn);
int tc_error_take();

// seeded synthetic bytes (parpar_gb300/synth.py layout); byteOffset (a
// multiple of 8) selects a window of each row's byte stream
int synth_fill(void* dst, size_t pitchBytes, unsigned nRows, size_t rowBytes, uint64_t seed, uint64_t first, cudaStream_t st,
               uint64_t byteOffset = 0);

// bounded-wait self-test (k_comb.cu): a wait that nothing completes gives up
// after `polls` polls and sets the multiply-accumulate error flag
int wait_selftest(unsigned polls, int* gaveUp, double* seconds);
// file MD5 with each chain's bytes staged into shared memory by bulk copies;
// table entry f's digest goes to dOut + 16 * dOutIndex[f] (f when null)
int file_md5_staged(const void* rows, size_t pitchBytes, unsigned nFiles, const uint64_t* dFileLen,
                    const uint32_t* dFirstRow, size_t sliceBytes, uint8_t* dOut, unsigned filesPerBlock, cudaStream_t st,
                    const uint32_t* dOutIndex = nullptr);
int hash_error_take();
// block-scaled 4-bit tcgen05 form (k_tc4.cu)
size_t tc4_scratch_bytes(unsigned R, unsigned nIn, size_t nWords);
// scratch for word chunks of at most aChunkBytes of expanded input planes
size_t tc4_scratch_chunked_bytes(unsigned R, unsigned nIn, size_t nWords, size_t aChunkBytes);
int tc4_muladd(const uint16_t* in, size_t inPitch, unsigned nIn, const uint16_t* coeff, uint16_t* rec, size_t recPitch,
               unsigned R, size_t nWords, int accumulate, void* scratch, size_t scratchBytes, cudaStream_t st);
int tc4_error_take();
int tc4_mma_rate(double* macsPerSec, cudaStream_t st);
int set_tc4_shape(int shape);
int set_tc4_group(int groupM);
unsigned tc4_launches(unsigned R, unsigned nIn, size_t nWords, size_t scratchBytes);
int tc4_shape_for(unsigned kBlocks);
} // namespace p2c
