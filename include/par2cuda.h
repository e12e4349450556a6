/*
 * par2cuda — C ABI of the GB300 (sm_103a) PAR2 recovery backend.
 *
 * One handle = one backend instance on one CUDA device, the counterpart of a
 * PAR2ProcOCL / PAR2ProcCPU object behind ParPar's backend plugin interface
 * IPAR2ProcBackend (gf16/controller.h:77-217).  Each entry point below names
 * the reference member it replaces.  The C++ adapter class PAR2ProcCUDA
 * (parpar_gb300/adapter/controller_cuda.{h,cpp}, which becomes
 * gf16/controller_cuda.{h,cpp} in a ParPar tree) derives from IPAR2ProcBackend
 * and forwards its virtuals to these functions, so PAR2Proc
 * (gf16/controller.cpp) and the node addon (src/gf.cc) drive it unchanged.
 *
 * Conventions
 *  - Plain pointers and sizes only.  Host buffers may be pageable or pinned;
 *    pinned (cudaHostAlloc / cudaHostRegister) buffers are copied directly.
 *  - Return value: 0 = success, negative = error (the message is available
 *    from par2cuda_last_error() on the calling thread).  The reference's
 *    `bool false` results ("Failed to allocate memory", src/gf.cc:351-354)
 *    map to a negative return.
 *  - Completion callbacks run on a backend-owned thread, in submission order
 *    per callback kind.  Under libuv the adapter re-posts them to the loop
 *    with ThreadNotifyQueue (gf16/threadqueue.h), as the OpenCL backend does.
 *  - Buffers passed to par2cuda_add_input are borrowed until its callback has
 *    run (the reference's future/callback contract, gf16/controller_cpu.cpp:283-331).
 *  - Output corruption is reported as valid = 0 in the get_output callback,
 *    never as an error (gf16/controller_cpu.cpp:423-443, src/gf.cc:680-692).
 *  - Slice sizes are byte counts of the current slice chunk: even, >= 2
 *    (src/gf.cc:262, gf16/controller.cpp:76-78).
 */
#ifndef PAR2CUDA_H
#define PAR2CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct par2cuda_ctx par2cuda_ctx;

/* status / verdict callback: status >= 0 on success (get_output: 1 = checksum
 * valid, 0 = invalid), negative on error */
typedef void (*par2cuda_done_fn)(void* user, int status);
/* batch-completion progress callback (IPAR2ProcBackend::progressCb,
 * gf16/controller.h:93, called from _notifyProc gf16/controller_cpu.cpp:627-645) */
typedef void (*par2cuda_progress_fn)(void* user, unsigned numInputs);

/* canAdd() results — PAR2ProcBackendAddResult, gf16/controller.h:38-43 */
enum { PAR2CUDA_ADD_OK = 0, PAR2CUDA_ADD_OK_BUSY = 1, PAR2CUDA_ADD_FULL = 2 };

/* multiply-accumulate kernels (the Galois16OCLMethods analogue, gf16/controller_ocl.h:15-31) */
enum {
	PAR2CUDA_METHOD_AUTO = 0,
	PAR2CUDA_METHOD_COMB = 1,   /* shared-memory XOR-combination tables (default) */
	PAR2CUDA_METHOD_XOR = 2,    /* LOP3 over 16 bit planes (per-coefficient-bit masks) */
	PAR2CUDA_METHOD_NIBBLE = 3, /* shared-memory split-nibble tables */
	PAR2CUDA_METHOD_TENSOR = 4, /* tcgen05 GF(2) bit-matrix product (e4m3 0/1, fp32 accumulators) */
	PAR2CUDA_METHOD_TENSOR_FP4 = 5 /* tcgen05 block-scaled 4-bit (mxf4) GF(2) product, TMA-fed; device level only */
};

typedef struct par2cuda_info {
	int device;
	char device_name[128];
	char method_desc[64];        /* GetInfo "method_desc" (src/gf.cc:527-568) */
	unsigned staging_count;      /* "staging_count" */
	unsigned staging_size;       /* "staging_size" = input batch size */
	unsigned min_staging_size;
	size_t chunk_size;           /* "chunk_size": bytes per kernel tile column (128) */
	size_t slice_mem;            /* "slice_mem": device bytes per slice row (pitch) */
	size_t slice_size;           /* current slice chunk size */
	unsigned num_output_slices;  /* "num_output_slices" */
	unsigned batches_started;    /* getBatchesStarted() gf16/controller.h:208-210 */
	size_t device_bytes;         /* device memory held by this backend */
} par2cuda_info;

/* Library version string. */
const char* par2cuda_version(void);
/* Message of the last failed call on this thread. */
const char* par2cuda_last_error(void);
/* Number of visible CUDA devices (negative on error) — the getDevices()
 * analogue of PAR2ProcOCL (gf16/controller_ocl.h:173). */
int par2cuda_device_count(void);

/* Constructor: PAR2ProcOCL(loop, platformId, deviceId, stagingAreas)
 * gf16/controller_ocl.h:188; stagingAreas as parsed in src/gf.cc:326-330. */
int par2cuda_create(int device, unsigned staging_areas, par2cuda_ctx** out);
/* init(method, targetInputBatch, ...) gf16/controller_ocl.h:191 /
 * PAR2ProcCPU::init gf16/controller_cpu.cpp:79-115.  input_batch = 0 picks a
 * default from the slice size.  Call after par2cuda_set_slice_size. */
int par2cuda_init(par2cuda_ctx* ctx, int method, unsigned input_batch);
/* setSliceSize(size) gf16/controller.h:160 */
int par2cuda_set_slice_size(par2cuda_ctx* ctx, size_t size);
/* setCurrentSliceSize(size) gf16/controller.h:166 (chunked passes,
 * gf16/controller.cpp:87-115, lib/par2.js:847-867) */
int par2cuda_set_current_slice_size(par2cuda_ctx* ctx, size_t size);
/* setRecoverySlices(numSlices, exponents) gf16/controller.h:167; exponents
 * may be NULL when every input is added with explicit coefficients */
int par2cuda_set_recovery_slices(par2cuda_ctx* ctx, unsigned num_slices, const uint16_t* exponents);
/* setMinInputBatchSize(size) gf16/controller.h:212-214 */
int par2cuda_set_min_input_batch(par2cuda_ctx* ctx, unsigned size);
/* setProgressCb gf16/controller.h:162-164 */
int par2cuda_set_progress_cb(par2cuda_ctx* ctx, par2cuda_progress_fn fn, void* user);

/* canAdd() gf16/controller.h:168 -> PAR2CUDA_ADD_* (negative on error) */
int par2cuda_can_add(par2cuda_ctx* ctx);
/* waitForAdd() gf16/controller.h:194 (blocks until canAdd() != FULL) */
int par2cuda_wait_for_add(par2cuda_ctx* ctx);
/* addInput(buffer, size, inputNum, flush[, cb]) gf16/controller.h:169;
 * size <= current slice size, shorter inputs are zero-padded;
 * input_num 0..32767 (src/gf.cc:587).  cb(user, 0) once `buffer` is free.
 * Returns 1 when this call submitted a batch (the controller's active batch
 * count goes up; the progress callback fires when it completes), 0 otherwise.
 * The same holds for par2cuda_add_input_coeffs, par2cuda_dummy_input and
 * par2cuda_flush. */
int par2cuda_add_input(par2cuda_ctx* ctx, const void* buffer, size_t size, uint16_t input_num, int flush,
                       par2cuda_done_fn cb, void* user);
/* addInput(buffer, size, coeffs, flush[, cb]) gf16/controller.h:170;
 * coeffs[r] = coefficient of this input for recovery slice r */
int par2cuda_add_input_coeffs(par2cuda_ctx* ctx, const void* buffer, size_t size, const uint16_t* coeffs,
                              int flush, par2cuda_done_fn cb, void* user);
/* dummyInput(inputNum, flush) gf16/controller.h:171 (benchmarking: counts an
 * input without transferring data) */
int par2cuda_dummy_input(par2cuda_ctx* ctx, uint16_t input_num, int flush);
/* fillInput(buffer) gf16/controller.h:172 (benchmarking: loads staging
 * without computing); returns 1 once every staging area has been filled */
int par2cuda_fill_input(par2cuda_ctx* ctx, const void* buffer);
/* flush() gf16/controller.h:173 */
int par2cuda_flush(par2cuda_ctx* ctx);
/* endInput() gf16/controller.h:175-179: flushes, and cb(user, 0) runs once
 * every batch has been processed (processing_finished, controller.h:192) */
int par2cuda_end_input(par2cuda_ctx* ctx, par2cuda_done_fn cb, void* user);
/* getOutput(index, output[, cb(valid)]) gf16/controller.h:185; `output`
 * holds >= current slice size bytes (src/gf.cc:668-669) */
int par2cuda_get_output(par2cuda_ctx* ctx, unsigned index, void* output, par2cuda_done_fn cb, void* user);
/* The `valid` of getOutput (gf16/controller.h:185, the bool its future
 * resolves to) read synchronously: 1 = checksum valid, 0 = invalid, negative
 * on error.  Waits for queued work (par2cuda_sync) and is meaningful once
 * end_input has been issued; lets a caller copy outputs without a callback
 * per slice. */
int par2cuda_output_valid(par2cuda_ctx* ctx, unsigned index);
/* discardOutput() gf16/controller.h:186-188: next batch overwrites */
int par2cuda_discard_output(par2cuda_ctx* ctx);
/* _hasAdded() gf16/controller.h:189-191 */
int par2cuda_has_added(par2cuda_ctx* ctx);
/* isEmpty() gf16/controller.h:182-184 */
int par2cuda_is_empty(par2cuda_ctx* ctx);
/* Blocks until every queued transfer, batch and callback has completed. */
int par2cuda_sync(par2cuda_ctx* ctx);
/* freeProcessingMem() gf16/controller.h:203 */
int par2cuda_free_processing_mem(par2cuda_ctx* ctx);
/* GfProc.info() fields, src/gf.cc:527-568 */
int par2cuda_info_get(par2cuda_ctx* ctx, par2cuda_info* out);
/* deinit() + destructor, gf16/controller.h:197-202 */
int par2cuda_destroy(par2cuda_ctx* ctx);

/* ---- device-level entry points (device pointers, caller's stream) ----
 * The kernels of the backend above, for callers that keep slices resident
 * on the GPU (the batched and serving paths).  `stream` is a cudaStream_t. */

/* Bytes between rows the backend uses for a slice of `slice_bytes`: the data
 * padded to 8 bytes, an 8-byte checksum block, rounded up to 128 bytes. */
size_t par2cuda_row_pitch_bytes(size_t slice_bytes);
/* Coefficient of input `input_num` for recovery exponent `exponent`
 * (gfmat_coeff, gf16/gfmat_coeff.c:75-77). */
uint16_t par2cuda_coeff(uint16_t input_num, uint16_t exponent);
/* CTA shape of the comb kernel for every later call in this process (the
 * autotuner's knob): 0 = chosen from the number of recovery rows, 1..9 = a
 * fixed (rows per warp x warps) shape; 10..15 = warp-specialised shapes
 * (4 table-building warps + 8 or 12 lookup warps, 2 or 4 words per lane);
 * 16..25 = warp-specialised shapes with two 8-input tables per ring slot
 * (20: one table, same prefetching builders); 26..28 = the same with the
 * builder warpgroup's registers moved to the lookup warps (84, 72 and 96
 * rows).  Returns the previous setting. */
int par2cuda_set_comb_shape(int shape);
/* Tile shape of the block-scaled 4-bit tensor method for every later call in
 * this process (the autotuner's knob): 0 = chosen from the number of inputs,
 * 1 = 128 words x 16 recovery slices with one TMEM accumulator, 2 = 128 words
 * x 12 recovery slices with two accumulators (a tile's read-out overlaps the
 * next tile's MMAs).  Returns the previous setting.  No counterpart in the
 * reference. */
int par2cuda_set_tc4_shape(int shape);
/* Raster group of the tensor_fp4 GEMM for every later call in this process
 * (the autotuner's knob): the number of 128-word tiles that walk the recovery
 * tiles together; 0 = chosen from the input count (as many as keep their
 * expanded input planes in about 48 MiB of L2).  Returns the previous
 * setting.  No counterpart in the reference. */
int par2cuda_set_tc4_group(int word_tiles);
/* The tile shape (1 or 2) the next tensor_fp4 call with num_in inputs will use. */
int par2cuda_tc4_shape_for(unsigned num_in);
/* Measures the rate (bytes/s) of one MD5 stream on one GPU thread with its
 * data in registers (about 0.1 s): the dependency-chain ceiling of the
 * one-stream-per-thread hash kernels (file MD5, IFSC, recovery-packet MD5).
 * No counterpart in the reference. */
int par2cuda_md5_chain_rate(double* bytes_per_s, void* stream);
/* The comb CTA shape the next multiply-accumulate with num_rec recovery rows
 * will use (the set_comb_shape setting, else the automatic choice). */
int par2cuda_comb_shape_for(unsigned num_rec);
/* Measures the current device's three-input LOP3 throughput (ops/s) with a
 * calibration kernel at full occupancy (about 0.1 s): the denominator of the
 * integer-ALU roofline (2 LOP3 per word multiply-accumulate).  No counterpart
 * in the reference. */
int par2cuda_lop3_rate(double* ops_per_s, void* stream);
/* Reads and clears the device-side error flags of the multiply-accumulate and
 * staged hash kernels: 1 when a bounded wait inside a kernel gave up (its
 * results are then invalid), 0 otherwise, negative if a flag could not be
 * read. */
int par2cuda_device_error(void);
/* Self-test of the kernels' bounded waits (no counterpart in the reference):
 * one warp waits, with the multiply-accumulate kernels' own wait helper and a
 * limit of `polls` (1..2^22) polls, on an mbarrier that nothing arrives on.
 * The wait gives up, sets the flag par2cuda_device_error() reports, and the
 * kernel returns; *gave_up = 1 then, *seconds = the kernel's duration.  The
 * context stays usable.  The kernels themselves use 2^22 polls. */
int par2cuda_wait_selftest(unsigned polls, int* gave_up, double* seconds);
/* Scratch bytes par2cuda_muladd needs for (num_rec, num_in). */
size_t par2cuda_muladd_scratch_bytes(unsigned num_rec, unsigned num_in);
/* Scratch bytes par2cuda_muladd needs for method PAR2CUDA_METHOD_TENSOR_FP4:
 * a 1 KiB header (the GEMM's tile counter, reset by every call), the
 * coefficient bit matrix (16 * roundup(num_rec, 48) rows of
 * roundup(num_in, 16) * 8 bytes) and the 4-bit input planes of a chunk of at
 * most 1 GiB of words (less scratch = smaller chunks; at least one 128-word
 * tile).  No counterpart in the reference. */
size_t par2cuda_tensor_fp4_scratch_bytes(unsigned num_rec, unsigned num_in, size_t n_words);
/* Measures the tensor pipe's rate (binary multiply-accumulates per second)
 * for the MMA of PAR2CUDA_METHOD_TENSOR_FP4 (M=128, N=256, K=64, mxf4) with one
 * CTA per SM issuing MMAs on shared-memory operands (about 0.1 s): the
 * roofline denominator of that method.  No counterpart in the reference. */
int par2cuda_tensor_fp4_rate(double* macs_per_s, void* stream);
/* The number of kernel launches one par2cuda_muladd call with these
 * arguments makes (the tensor_fp4 method: one per word chunk of expanded
 * input planes and GEMM, plus the coefficient expansion).  No counterpart in
 * the reference. */
int par2cuda_muladd_launches(unsigned num_rec, unsigned num_in, size_t n_words, int method, size_t scratch_bytes);
/* rec[r][0..n_words) (^)= sum_i coeff[r*num_in + i] * in[i][0..n_words),
 * the run_kernel body (gf16/controller_cpu.cpp:488-515).  Pitches are in
 * 16-bit words (even); rows must be readable/writable up to
 * roundup(n_words, 64) words (par2cuda_row_pitch_bytes gives such rows).
 * accumulate = 0 overwrites rec (processingAdd false). */
int par2cuda_muladd(const uint16_t* d_in, size_t in_pitch_words, unsigned num_in,
                    const uint16_t* d_coeff, uint16_t* d_rec, size_t rec_pitch_words, unsigned num_rec,
                    size_t n_words, int accumulate, int method, void* d_scratch, size_t scratch_bytes,
                    void* stream);
/* par2cuda_muladd with the comb method, for callers that cannot supply or
 * allocate scratch memory (a fixed device-memory budget, or a submission loop
 * that must not call cudaMalloc because an allocation may synchronise the
 * device).  No counterpart in the reference.  The scratch is a 4 MiB array
 * inside the library on each device that loads it, so it requires
 * num_rec * ceil(num_in / 8) <= 262144 (larger calls are rejected with an
 * error; split the inputs over several calls with accumulate = 1).  It
 * allocates nothing.  The first call on a device looks up the array's address
 * (make it before any stream capture) and keeps it for the life of the
 * process: do not use this entry point across a cudaDeviceReset or anything
 * else that destroys and recreates the device's primary context, which can
 * move the array.  All calls share the array: calls that overlap on the GPU
 * race, so order them on one stream or with events. */
int par2cuda_muladd_noalloc(const uint16_t* d_in, size_t in_pitch_words, unsigned num_in,
                            const uint16_t* d_coeff, uint16_t* d_rec, size_t rec_pitch_words, unsigned num_rec,
                            size_t n_words, int accumulate, void* stream);
/* Zero-pads rows past lens[i] bytes and writes the internal checksum block
 * of each row (gf16_cksum_copy, gf16/gf16_cksum_base.h:32-46), or with
 * verify = 1 compares it into d_flags[i] (gf16_cksum_copy_check :48-60).
 * d_lens may be NULL (every row is slice_bytes long).  d_scratch: 8 bytes per row. */
int par2cuda_rows_checksum(uint16_t* d_rows, size_t pitch_words, unsigned num_rows, const uint32_t* d_lens,
                           size_t slice_bytes, int verify, uint8_t* d_flags, void* d_scratch, void* stream);
/* IFSC entries (hasher/hasher_base.h:154-176): for each row i, MD5 of its
 * first d_lens[i] bytes zero-padded to slice_bytes, then CRC32 of the same
 * (little-endian), 20 bytes per row into d_ifsc.  One GPU thread per row.
 * d_lens may be NULL (full rows).  pitch_bytes: multiple of 16. */
int par2cuda_slice_hash(const void* d_rows, size_t pitch_bytes, unsigned num_rows, const uint32_t* d_lens,
                        size_t slice_bytes, uint8_t* d_ifsc, void* stream);
/* File MD5s (HasherInput::end, hasher/hasher_base.h:178-186): file f is the
 * d_file_len[f] bytes held by consecutive rows from d_first_row[f], each row
 * holding slice_bytes of it.  One GPU thread per file; 16 bytes per file. */
int par2cuda_file_md5(const void* d_rows, size_t pitch_bytes, unsigned num_files, const uint64_t* d_file_len,
                      const uint32_t* d_first_row, size_t slice_bytes, uint8_t* d_md5, void* stream);
/* par2cuda_file_md5 with 32 files per warp instead of one per block: each
 * chain runs ~6 % slower, but the hashes occupy ceil(num_files/32) blocks,
 * leaving the other SMs to concurrent work (several jobs in flight).  Same
 * results.  No counterpart in the reference. */
int par2cuda_file_md5_packed(const void* d_rows, size_t pitch_bytes, unsigned num_files, const uint64_t* d_file_len,
                             const uint32_t* d_first_row, size_t slice_bytes, uint8_t* d_md5, void* stream);
/* par2cuda_file_md5 with `files_per_block` files (1, or a multiple of 32 up to
 * 512) per block: the file MD5 chains of several jobs in flight (the rows of
 * all of them reachable from d_rows through d_first_row) held on as few SMs as
 * possible, so that the other SMs stay free for the jobs' contractions.  Same
 * results.  No counterpart in the reference. */
int par2cuda_file_md5_pooled(const void* d_rows, size_t pitch_bytes, unsigned num_files, const uint64_t* d_file_len,
                             const uint32_t* d_first_row, size_t slice_bytes, uint8_t* d_md5, unsigned files_per_block,
                             void* stream);
/* MD5 of (d_prefix[i*prefix_len .. +prefix_len) ++ first data_len bytes of
 * row i) for each row: the recovery-packet hash that MD5Multi computes
 * (src/gf.cc:1075-1219, lib/par2.js:243-335).  One GPU thread per row. */
int par2cuda_rows_md5(const void* d_rows, size_t pitch_bytes, unsigned num_rows, size_t data_len,
                      const uint8_t* d_prefix, unsigned prefix_len, uint8_t* d_md5, void* stream);
/* par2cuda_file_md5 with each file's bytes staged into shared memory ahead of
 * its hash chain by bulk asynchronous copies (TMA, three 1 KiB chunks in
 * flight per file), so the serial chain never waits on a cache miss while
 * other work streams through L2.  files_per_block: 32 or 64.  Requires
 * slice_bytes % 64 == 0 and 16-byte aligned rows.  A bounded wait that gives
 * up sets the flag par2cuda_device_error() reports.  Same results.  No
 * counterpart in the reference. */
int par2cuda_file_md5_staged(const void* d_rows, size_t pitch_bytes, unsigned num_files, const uint64_t* d_file_len,
                             const uint32_t* d_first_row, size_t slice_bytes, uint8_t* d_md5, unsigned files_per_block,
                             void* stream);
/* par2cuda_file_md5_staged over any subset of files, in any order: table
 * entry f's digest is written to d_md5 + 16 * d_out_index[f] (to d_md5 +
 * 16 * f when d_out_index is NULL).  A job stream hashes its largest files
 * first, as soon as their rows have landed, and the rest later, each digest
 * in its file's place.  No counterpart in the reference. */
int par2cuda_file_md5_staged_indexed(const void* d_rows, size_t pitch_bytes, unsigned num_files,
                                     const uint64_t* d_file_len, const uint32_t* d_first_row,
                                     const uint32_t* d_out_index, size_t slice_bytes, uint8_t* d_md5,
                                     unsigned files_per_block, void* stream);
/* Copies num_rows rows of row_bytes bytes between host and device memory (or
 * within either) with one 2-D copy on `stream`: the H2D of input slices into
 * the backend's pitched rows, the D2H of recovery rows into packed host
 * slices.  Asynchronous with respect to the host for pinned host memory. */
int par2cuda_copy_rows(void* dst, size_t dst_pitch, const void* src, size_t src_pitch, size_t row_bytes,
                       unsigned num_rows, void* stream);
/* Seeded synthetic bytes (same bytes as parpar_gb300/synth.py). */
int par2cuda_synth_fill(void* d_dst, size_t pitch_bytes, unsigned num_rows, size_t row_bytes,
                        uint64_t seed, uint64_t first_index, void* stream);
/* The same bytes for the window [byte_offset, byte_offset + row_bytes) of each
 * row's stream (byte_offset a multiple of 8): slice data for chunked passes. */
int par2cuda_synth_fill_at(void* d_dst, size_t pitch_bytes, unsigned num_rows, size_t row_bytes,
                           uint64_t seed, uint64_t first_index, uint64_t byte_offset, void* stream);

/* ---- batched multiply-accumulate over many jobs (one persistent launch) ----
 * The reference processes one PAR2 job per controller; a GPU is only busy
 * when many jobs share it, so this entry point runs the multiply-accumulate of
 * many jobs (each with its own inputs, coefficients and recovery rows) in one
 * persistent launch.  A job's work is split into units of (64-word tile x
 * recovery block); CTAs take units from *d_counter (reset by the call), largest
 * job first when the array is sorted that way. */
typedef struct par2cuda_batch_job {
	const uint16_t* d_in;        /* input rows */
	size_t in_pitch_words;
	unsigned num_in;
	const void* d_index;         /* index bytes from par2cuda_coeff_index */
	uint16_t* d_rec;             /* recovery rows */
	size_t rec_pitch_words;
	unsigned num_rec;
	int accumulate;
	unsigned long long unit_base; /* sum of par2cuda_batch_units() of the jobs before it */
} par2cuda_batch_job;
/* Bytes of index data for a job (num_rec x ceil(num_in/8) x 16). */
size_t par2cuda_coeff_index_bytes(unsigned num_rec, unsigned num_in);
/* Index bytes of a job from its coefficient matrix d_coeff[num_rec][num_in]. */
int par2cuda_coeff_index(const uint16_t* d_coeff, unsigned num_rec, unsigned num_in, void* d_index, void* stream);
/* Index bytes of a PAR2 job computed on the device from its input numbers
 * d_input_nums[num_in] and recovery exponents d_exponents[num_rec]
 * (set_coeffs, gf16/controller_cpu.cpp:372-379, without a host matrix). */
int par2cuda_par2_index(const uint16_t* d_input_nums, unsigned num_in, const uint16_t* d_exponents, unsigned num_rec,
                        void* d_index, void* stream);
/* The PAR2 coefficient matrix d_coeff[num_rec][num_in] itself, computed on
 * the device the same way (gfmat_coeff, gf16/gfmat_coeff.c:60-77), for the
 * multiply methods of par2cuda_muladd that read coefficients. */
int par2cuda_par2_coeffs(const uint16_t* d_input_nums, unsigned num_in, const uint16_t* d_exponents, unsigned num_rec,
                         uint16_t* d_coeff, void* stream);
/* Work units of a job with num_rec rows of n_words words for batched CTA
 * shape 1..7 (1..4: one-phase, 8 x {1,4,8,12} recovery rows per unit; 5..7:
 * paired tables, {72,64,32} rows per unit); 0 for an unknown shape. */
unsigned long long par2cuda_batch_units(unsigned num_rec, size_t n_words, int shape);
/* One persistent launch over d_jobs[0..num_jobs) (device array). */
int par2cuda_batch_muladd(const par2cuda_batch_job* d_jobs, unsigned num_jobs, unsigned long long total_units,
                          unsigned long long* d_counter, int shape, void* stream);
/* Multiply-accumulate of one job from index bytes prepared once
 * (par2cuda_coeff_index or par2cuda_par2_index), as a grid launch of the
 * automatic comb shape: d_rec[r] (^)= sum_i c(r,i) d_in[i] over n_words words.
 * Pitches are in 16-bit words and at least roundup(n_words, 64).  No
 * counterpart in the reference (its kernels take coefficients per call); it
 * serves callers that keep a job's index resident across chunks. */
int par2cuda_muladd_index(const uint16_t* d_in, size_t in_pitch_words, unsigned num_in, const void* d_index,
                          uint16_t* d_rec, size_t rec_pitch_words, unsigned num_rec, size_t n_words, int accumulate,
                          void* stream);

#ifdef __cplusplus
}
#endif

#endif /* PAR2CUDA_H */
