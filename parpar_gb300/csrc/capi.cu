// extern "C" entry points of include/par2cuda.h.
#include "engine.h"

#include <cstddef>
#include <cstring>
#include <new>

namespace p2c { const uint16_t* host_input_logs(); }

struct par2cuda_ctx {
	p2c::Engine* eng;
};

#define P2C_CTX_CHECK(ctx) do { if(!(ctx) || !(ctx)->eng) { p2c::set_error("null handle"); return -1; } } while(0)

extern "C" {

const char* par2cuda_version(void) { return "par2cuda 0.1 (sm_103a)"; }
const char* par2cuda_last_error(void) { return p2c::get_error(); }

int par2cuda_device_count(void) {
	int n = 0;
	cudaError_t e = cudaGetDeviceCount(&n);
	if(e != cudaSuccess) { p2c::set_error("cudaGetDeviceCount: %s", cudaGetErrorString(e)); return -1; }
	return n;
}

int par2cuda_create(int device, unsigned staging_areas, par2cuda_ctx** out) {
	if(!out) { p2c::set_error("null output handle"); return -1; }
	*out = nullptr;
	if(staging_areas < 1 || staging_areas > 32768) { p2c::set_error("staging area count %u is invalid", staging_areas); return -1; }
	int n = par2cuda_device_count();
	if(n < 0) return -1;
	if(device < 0 || device >= n) { p2c::set_error("device %d not present (%d visible)", device, n); return -1; }
	auto* ctx = new(std::nothrow) par2cuda_ctx;
	if(!ctx) { p2c::set_error("out of host memory"); return -1; }
	ctx->eng = new(std::nothrow) p2c::Engine(device, staging_areas);
	if(!ctx->eng || ctx->eng->start()) {
		delete ctx->eng;
		delete ctx;
		return -1;
	}
	*out = ctx;
	return 0;
}

int par2cuda_init(par2cuda_ctx* ctx, int method, unsigned input_batch) {
	P2C_CTX_CHECK(ctx);
	return ctx->eng->init(method, input_batch);
}
int par2cuda_set_slice_size(par2cuda_ctx* ctx, size_t size) { P2C_CTX_CHECK(ctx); return ctx->eng->set_slice_size(size); }
int par2cuda_set_current_slice_size(par2cuda_ctx* ctx, size_t size) { P2C_CTX_CHECK(ctx); return ctx->eng->set_current_slice_size(size); }
int par2cuda_set_recovery_slices(par2cuda_ctx* ctx, unsigned n, const uint16_t* exps) {
	P2C_CTX_CHECK(ctx);
	if(n > 65534) { p2c::set_error("too many recovery slices (%u)", n); return -1; }
	if(exps) for(unsigned i = 0; i < n; i++) if(exps[i] > 65534) { p2c::set_error("invalid recovery exponent %u", exps[i]); return -1; }
	return ctx->eng->set_recovery_slices(n, exps);
}
int par2cuda_set_min_input_batch(par2cuda_ctx* ctx, unsigned size) { P2C_CTX_CHECK(ctx); ctx->eng->set_min_input_batch(size); return 0; }
int par2cuda_set_progress_cb(par2cuda_ctx* ctx, par2cuda_progress_fn fn, void* user) { P2C_CTX_CHECK(ctx); ctx->eng->set_progress(fn, user); return 0; }
int par2cuda_can_add(par2cuda_ctx* ctx) { P2C_CTX_CHECK(ctx); return ctx->eng->can_add(); }
int par2cuda_wait_for_add(par2cuda_ctx* ctx) { P2C_CTX_CHECK(ctx); return ctx->eng->wait_for_add(); }
int par2cuda_add_input(par2cuda_ctx* ctx, const void* buffer, size_t size, uint16_t input_num, int flush,
                       par2cuda_done_fn cb, void* user) {
	P2C_CTX_CHECK(ctx);
	if(size && !buffer) { p2c::set_error("null input buffer"); return -1; }
	return ctx->eng->add_input(buffer, size, input_num, nullptr, flush != 0, cb, user);
}
int par2cuda_add_input_coeffs(par2cuda_ctx* ctx, const void* buffer, size_t size, const uint16_t* coeffs, int flush,
                              par2cuda_done_fn cb, void* user) {
	P2C_CTX_CHECK(ctx);
	if((size && !buffer) || !coeffs) { p2c::set_error("null input buffer or coefficients"); return -1; }
	return ctx->eng->add_input(buffer, size, 0, coeffs, flush != 0, cb, user);
}
int par2cuda_dummy_input(par2cuda_ctx* ctx, uint16_t input_num, int flush) {
	P2C_CTX_CHECK(ctx);
	return ctx->eng->add_input(nullptr, 0, input_num, nullptr, flush != 0, nullptr, nullptr, true);
}
int par2cuda_fill_input(par2cuda_ctx* ctx, const void* buffer) { P2C_CTX_CHECK(ctx); return ctx->eng->fill_input(buffer); }
int par2cuda_flush(par2cuda_ctx* ctx) { P2C_CTX_CHECK(ctx); return ctx->eng->flush(); }
int par2cuda_end_input(par2cuda_ctx* ctx, par2cuda_done_fn cb, void* user) { P2C_CTX_CHECK(ctx); return ctx->eng->end_input(cb, user); }
int par2cuda_get_output(par2cuda_ctx* ctx, unsigned index, void* output, par2cuda_done_fn cb, void* user) {
	P2C_CTX_CHECK(ctx);
	if(!output) { p2c::set_error("null output buffer"); return -1; }
	return ctx->eng->get_output(index, output, cb, user);
}
int par2cuda_output_valid(par2cuda_ctx* ctx, unsigned index) { P2C_CTX_CHECK(ctx); return ctx->eng->output_valid(index); }
int par2cuda_discard_output(par2cuda_ctx* ctx) { P2C_CTX_CHECK(ctx); ctx->eng->discard_output(); return 0; }
int par2cuda_has_added(par2cuda_ctx* ctx) { P2C_CTX_CHECK(ctx); return ctx->eng->has_added() ? 1 : 0; }
int par2cuda_is_empty(par2cuda_ctx* ctx) { P2C_CTX_CHECK(ctx); return ctx->eng->is_empty() ? 1 : 0; }
int par2cuda_sync(par2cuda_ctx* ctx) { P2C_CTX_CHECK(ctx); return ctx->eng->sync(); }
int par2cuda_free_processing_mem(par2cuda_ctx* ctx) { P2C_CTX_CHECK(ctx); return ctx->eng->free_processing_mem(); }
int par2cuda_info_get(par2cuda_ctx* ctx, par2cuda_info* out) {
	P2C_CTX_CHECK(ctx);
	if(!out) { p2c::set_error("null info"); return -1; }
	return ctx->eng->info(out);
}
int par2cuda_destroy(par2cuda_ctx* ctx) {
	if(!ctx) return 0;
	delete ctx->eng;
	delete ctx;
	return 0;
}

// ---------------------------------------------------------------- device level
size_t par2cuda_row_pitch_bytes(size_t slice_bytes) { return p2c::row_pitch(slice_bytes) * 2; }

uint16_t par2cuda_coeff(uint16_t input_num, uint16_t exponent) {
	const uint16_t* logs = p2c::host_input_logs();
	uint32_t e = ((uint32_t)logs[input_num & 32767] * exponent) % 65535u;
	uint32_t n = 1;
	// 2^e by square-and-multiply in GF(2^16)
	uint32_t b = 2;
	while(e) {
		if(e & 1) {
			uint32_t p = 0, x = n;
			for(int i = 0; i < 16; i++) { if(b >> i & 1) p ^= x; x <<= 1; if(x & 0x10000) x ^= P2C_POLY; }
			n = p;
		}
		uint32_t p = 0, x = b;
		for(int i = 0; i < 16; i++) { if(b >> i & 1) p ^= x; x <<= 1; if(x & 0x10000) x ^= P2C_POLY; }
		b = p;
		e >>= 1;
	}
	return (uint16_t)n;
}

int par2cuda_set_comb_shape(int shape) {
	if(shape < 0 || shape > 28) { p2c::set_error("comb shape %d out of range 0..28", shape); return -1; }
	return p2c::set_comb_shape(shape);
}

int par2cuda_set_tc4_shape(int shape) {
	if(shape < 0 || shape > 2) { p2c::set_error("tensor_fp4 tile shape %d out of range 0..2", shape); return -1; }
	return p2c::set_tc4_shape(shape);
}

int par2cuda_set_tc4_group(int word_tiles) {
	if(word_tiles < 0 || word_tiles > 4096) { p2c::set_error("tensor_fp4 raster group %d out of range 0..4096", word_tiles); return -1; }
	return p2c::set_tc4_group(word_tiles);
}

int par2cuda_tc4_shape_for(unsigned num_in) { return p2c::tc4_shape_for((unsigned)((num_in + 15) / 16)); }

int par2cuda_md5_chain_rate(double* bytes_per_s, void* stream) {
	if(!bytes_per_s) { p2c::set_error("md5_chain_rate: null output"); return -1; }
	return p2c::md5_chain_rate(bytes_per_s, (cudaStream_t)stream);
}

int par2cuda_comb_shape_for(unsigned num_rec) { return p2c::comb_shape_for(num_rec); }

int par2cuda_lop3_rate(double* ops_per_s, void* stream) {
	if(!ops_per_s) { p2c::set_error("lop3_rate: null output"); return -1; }
	return p2c::lop3_rate(ops_per_s, (cudaStream_t)stream);
}

int par2cuda_wait_selftest(unsigned polls, int* gave_up, double* seconds) {
	if(polls == 0 || polls > (1u << 22)) { p2c::set_error("wait self-test: polls must be 1..2^22"); return -1; }
	return p2c::wait_selftest(polls, gave_up, seconds);
}

int par2cuda_device_error(void) {
	int a = p2c::comb_error_take(), b = p2c::tc_error_take(), c = p2c::hash_error_take(), d = p2c::tc4_error_take();
	if(a < 0 || b < 0 || c < 0 || d < 0) return -1;
	return (a || b || c || d) ? 1 : 0;
}

size_t par2cuda_muladd_scratch_bytes(unsigned num_rec, unsigned num_in) {
	// enough for every method: comb index bytes, tensor bit-matrix rows
	return p2c::round_up(std::max(p2c::idx_bytes(num_rec, num_in), p2c::tc_scratch_bytes(num_rec, num_in)), 256);
}

int par2cuda_tensor_fp4_rate(double* macs_per_s, void* stream) {
	if(!macs_per_s) { p2c::set_error("tensor_fp4_rate: null output"); return -1; }
	return p2c::tc4_mma_rate(macs_per_s, (cudaStream_t)stream);
}

size_t par2cuda_tensor_fp4_scratch_bytes(unsigned num_rec, unsigned num_in, size_t n_words) {
	return p2c::tc4_scratch_bytes(num_rec, num_in, n_words);
}

int par2cuda_muladd_launches(unsigned num_rec, unsigned num_in, size_t n_words, int method, size_t scratch_bytes) {
	if(!num_rec || !n_words) return 0;
	switch(method) {
	case PAR2CUDA_METHOD_XOR: case PAR2CUDA_METHOD_NIBBLE: return 1;
	case PAR2CUDA_METHOD_TENSOR: return 2;
	case PAR2CUDA_METHOD_TENSOR_FP4: return (int)p2c::tc4_launches(num_rec, num_in, n_words, scratch_bytes);
	case PAR2CUDA_METHOD_AUTO: case PAR2CUDA_METHOD_COMB: return 2;
	default: p2c::set_error("unknown method %d", method); return -1;
	}
}

int par2cuda_muladd(const uint16_t* d_in, size_t in_pitch_words, unsigned num_in, const uint16_t* d_coeff,
                    uint16_t* d_rec, size_t rec_pitch_words, unsigned num_rec, size_t n_words, int accumulate,
                    int method, void* d_scratch, size_t scratch_bytes, void* stream) {
	cudaStream_t st = (cudaStream_t)stream;
	if((in_pitch_words & 1) || (rec_pitch_words & 1)) { p2c::set_error("row pitches must be even (whole u32 pairs)"); return -1; }
	if(method == PAR2CUDA_METHOD_XOR)
		return p2c::xor_planes_muladd(d_in, in_pitch_words, num_in, d_coeff, d_rec, rec_pitch_words, num_rec, n_words, accumulate, st);
	if(method == PAR2CUDA_METHOD_TENSOR_FP4)
		return p2c::tc4_muladd(d_in, in_pitch_words, num_in, d_coeff, d_rec, rec_pitch_words, num_rec, n_words, accumulate,
		                       d_scratch, scratch_bytes, st);
	if(method == PAR2CUDA_METHOD_TENSOR)
		return p2c::tc_muladd(d_in, in_pitch_words, num_in, d_coeff, d_rec, rec_pitch_words, num_rec, n_words, accumulate, true,
		                      d_scratch, scratch_bytes, st);
	if(method == PAR2CUDA_METHOD_NIBBLE) {
		int dev = 0;
		P2C_CUDA_TRY(cudaGetDevice(&dev));
		p2c::GfTables gt;
		if(p2c::gf_tables(dev, &gt)) return -1;
		return p2c::nibble_muladd_t(d_in, in_pitch_words, num_in, d_coeff, d_rec, rec_pitch_words, num_rec, n_words, accumulate, gt, st);
	}
	if(method != PAR2CUDA_METHOD_AUTO && method != PAR2CUDA_METHOD_COMB) { p2c::set_error("unknown method %d", method); return -1; }
	size_t need = par2cuda_muladd_scratch_bytes(num_rec, num_in);
	if(scratch_bytes < need || (!d_scratch && need)) { p2c::set_error("scratch of %zu bytes needed, %zu given", need, scratch_bytes); return -1; }
	uint4* idx = reinterpret_cast<uint4*>(d_scratch);
	if(p2c::coeff_to_idx(d_coeff, num_rec, num_in, idx, st)) return -1;
	return p2c::comb_muladd(d_in, in_pitch_words, num_in, idx, d_rec, rec_pitch_words, num_rec, n_words, accumulate, 0, st);
}

int par2cuda_rows_checksum(uint16_t* d_rows, size_t pitch_words, unsigned num_rows, const uint32_t* d_lens,
                           size_t slice_bytes, int verify, uint8_t* d_flags, void* d_scratch, void* stream) {
	int dev = 0;
	P2C_CUDA_TRY(cudaGetDevice(&dev));
	p2c::GfTables gt;
	if(p2c::gf_tables(dev, &gt)) return -1;
	if(verify && !d_flags) { p2c::set_error("verify needs d_flags"); return -1; }
	return p2c::rows_cksum(d_rows, pitch_words, num_rows, d_lens, slice_bytes, (unsigned long long*)d_scratch,
	                       verify, d_flags, gt, (cudaStream_t)stream);
}

int par2cuda_slice_hash(const void* d_rows, size_t pitch_bytes, unsigned num_rows, const uint32_t* d_lens,
                        size_t slice_bytes, uint8_t* d_ifsc, void* stream) {
	return p2c::slice_hash(d_rows, pitch_bytes, num_rows, d_lens, slice_bytes, d_ifsc, (cudaStream_t)stream);
}
int par2cuda_file_md5(const void* d_rows, size_t pitch_bytes, unsigned num_files, const uint64_t* d_file_len,
                      const uint32_t* d_first_row, size_t slice_bytes, uint8_t* d_md5, void* stream) {
	return p2c::file_md5(d_rows, pitch_bytes, num_files, d_file_len, d_first_row, slice_bytes, d_md5, (cudaStream_t)stream);
}
int par2cuda_file_md5_packed(const void* d_rows, size_t pitch_bytes, unsigned num_files, const uint64_t* d_file_len,
                             const uint32_t* d_first_row, size_t slice_bytes, uint8_t* d_md5, void* stream) {
	return p2c::file_md5(d_rows, pitch_bytes, num_files, d_file_len, d_first_row, slice_bytes, d_md5, (cudaStream_t)stream,
	                     32);
}
int par2cuda_file_md5_pooled(const void* d_rows, size_t pitch_bytes, unsigned num_files, const uint64_t* d_file_len,
                             const uint32_t* d_first_row, size_t slice_bytes, uint8_t* d_md5, unsigned files_per_block,
                             void* stream) {
	return p2c::file_md5(d_rows, pitch_bytes, num_files, d_file_len, d_first_row, slice_bytes, d_md5, (cudaStream_t)stream,
	                     files_per_block);
}
int par2cuda_rows_md5(const void* d_rows, size_t pitch_bytes, unsigned num_rows, size_t data_len,
                      const uint8_t* d_prefix, unsigned prefix_len, uint8_t* d_md5, void* stream) {
	return p2c::rows_md5(d_rows, pitch_bytes, num_rows, data_len, d_prefix, prefix_len, d_md5, (cudaStream_t)stream);
}

int par2cuda_synth_fill(void* d_dst, size_t pitch_bytes, unsigned num_rows, size_t row_bytes, uint64_t seed,
                        uint64_t first_index, void* stream) {
	return p2c::synth_fill(d_dst, pitch_bytes, num_rows, row_bytes, seed, first_index, (cudaStream_t)stream);
}

int par2cuda_synth_fill_at(void* d_dst, size_t pitch_bytes, unsigned num_rows, size_t row_bytes, uint64_t seed,
                           uint64_t first_index, uint64_t byte_offset, void* stream) {
	return p2c::synth_fill(d_dst, pitch_bytes, num_rows, row_bytes, seed, first_index, (cudaStream_t)stream, byte_offset);
}

int par2cuda_file_md5_staged(const void* d_rows, size_t pitch_bytes, unsigned num_files, const uint64_t* d_file_len,
                             const uint32_t* d_first_row, size_t slice_bytes, uint8_t* d_md5, unsigned files_per_block,
                             void* stream) {
	return p2c::file_md5_staged(d_rows, pitch_bytes, num_files, d_file_len, d_first_row, slice_bytes, d_md5,
	                            files_per_block, (cudaStream_t)stream);
}
int par2cuda_file_md5_staged_indexed(const void* d_rows, size_t pitch_bytes, unsigned num_files,
                                     const uint64_t* d_file_len, const uint32_t* d_first_row,
                                     const uint32_t* d_out_index, size_t slice_bytes, uint8_t* d_md5,
                                     unsigned files_per_block, void* stream) {
	return p2c::file_md5_staged(d_rows, pitch_bytes, num_files, d_file_len, d_first_row, slice_bytes, d_md5,
	                            files_per_block, (cudaStream_t)stream, d_out_index);
}
int par2cuda_copy_rows(void* dst, size_t dst_pitch, const void* src, size_t src_pitch, size_t row_bytes,
                       unsigned num_rows, void* stream) {
	if(!num_rows || !row_bytes) return 0;
	if(!dst || !src || dst_pitch < row_bytes || src_pitch < row_bytes) {
		p2c::set_error("copy_rows: null pointer or pitch below the row size");
		return -1;
	}
	cudaError_t e = cudaMemcpy2DAsync(dst, dst_pitch, src, src_pitch, row_bytes, num_rows, cudaMemcpyDefault,
	                                  (cudaStream_t)stream);
	if(e != cudaSuccess) { p2c::set_error("cudaMemcpy2DAsync: %s", cudaGetErrorString(e)); return -1; }
	return 0;
}

size_t par2cuda_coeff_index_bytes(unsigned num_rec, unsigned num_in) { return p2c::idx_bytes(num_rec, num_in); }

int par2cuda_coeff_index(const uint16_t* d_coeff, unsigned num_rec, unsigned num_in, void* d_index, void* stream) {
	return p2c::coeff_to_idx(d_coeff, num_rec, num_in, reinterpret_cast<uint4*>(d_index), (cudaStream_t)stream);
}

int par2cuda_par2_index(const uint16_t* d_input_nums, unsigned num_in, const uint16_t* d_exponents, unsigned num_rec,
                        void* d_index, void* stream) {
	int dev = 0;
	P2C_CUDA_TRY(cudaGetDevice(&dev));
	p2c::GfTables gt;
	if(p2c::gf_tables(dev, &gt)) return -1;
	return p2c::par2_idx(d_input_nums, d_exponents, num_rec, num_in, reinterpret_cast<uint4*>(d_index), gt, (cudaStream_t)stream);
}

int par2cuda_par2_coeffs(const uint16_t* d_input_nums, unsigned num_in, const uint16_t* d_exponents, unsigned num_rec,
                         uint16_t* d_coeff, void* stream) {
	int dev = 0;
	P2C_CUDA_TRY(cudaGetDevice(&dev));
	p2c::GfTables gt;
	if(p2c::gf_tables(dev, &gt)) return -1;
	return p2c::par2_coeffs(d_input_nums, d_exponents, num_rec, num_in, d_coeff, gt, (cudaStream_t)stream);
}

unsigned long long par2cuda_batch_units(unsigned num_rec, size_t n_words, int shape) {
	return p2c::comb_units(num_rec, n_words, shape);
}

static_assert(sizeof(par2cuda_batch_job) == sizeof(p2c::BatchJob), "batch job layout");
static_assert(offsetof(par2cuda_batch_job, unit_base) == offsetof(p2c::BatchJob, unitBase), "batch job layout");
static_assert(offsetof(par2cuda_batch_job, d_rec) == offsetof(p2c::BatchJob, rec), "batch job layout");

int par2cuda_batch_muladd(const par2cuda_batch_job* d_jobs, unsigned num_jobs, unsigned long long total_units,
                          unsigned long long* d_counter, int shape, void* stream) {
	if(!d_counter && total_units) { p2c::set_error("null work counter"); return -1; }
	return p2c::comb_batched(reinterpret_cast<const p2c::BatchJob*>(d_jobs), num_jobs, total_units, d_counter, shape,
	                         (cudaStream_t)stream);
}

int par2cuda_muladd_index(const uint16_t* d_in, size_t in_pitch_words, unsigned num_in, const void* d_index,
                          uint16_t* d_rec, size_t rec_pitch_words, unsigned num_rec, size_t n_words, int accumulate,
                          void* stream) {
	if(!num_rec || !n_words) return 0;
	if((!d_in && num_in) || !d_rec || (!d_index && num_in)) { p2c::set_error("muladd_index: null pointer"); return -1; }
	if(in_pitch_words < p2c::round_up(n_words, P2C_TILE_WORDS) || rec_pitch_words < p2c::round_up(n_words, P2C_TILE_WORDS)) {
		p2c::set_error("muladd_index: row pitch below roundup(n_words, 64)");
		return -1;
	}
	return p2c::comb_muladd(d_in, in_pitch_words, num_in, reinterpret_cast<const uint4*>(d_index), d_rec, rec_pitch_words,
	                        num_rec, n_words, accumulate, 0, (cudaStream_t)stream);
}

} // extern "C"
