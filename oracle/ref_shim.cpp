// Test infrastructure only: a thin C driver over the reference's own CPU
// implementation (ParPar's gf16/ controller + hasher), compiled in place from the
// reference sources by oracle/ref.mk into oracle/_ref/libparref.so.  It is
// used to pin the oracle restatement (oracle/par2_oracle.c) and to generate the
// golden fixtures under tests/golden/.  Nothing in the product links it.
//
// The driver follows the reference's own non-libuv usage pattern:
//   PAR2Proc + PAR2ProcCPU   gf16/controller.h:248-326, gf16/controller_cpu.h:20-145
//   waitForAdd/addInput/endInput/getOutput   gf16/controller.cpp:164-399
//   HasherInput update/getBlock/end          hasher/hasher_base.h:103-186
#include "gf16/controller.h"
#include "gf16/controller_cpu.h"
#include "gf16/gfmat_coeff.h"
extern "C" {
#include "gf16/gf16_cksum.h"
}
#include "hasher/hasher.h"

#include <chrono>
#include <cstring>
#include <string>
#include <vector>

static std::string g_method_name;

extern "C" {

uint16_t ref_gf_exp(uint16_t v) { gfmat_init(); return gf16_exp(v); }
uint16_t ref_input_log(uint16_t input) { gfmat_init(); return gfmat_input_log(input); }
uint16_t ref_coeff(uint16_t input, uint16_t exponent) { gfmat_init(); return gfmat_coeff(input, exponent); }

void ref_cksum_copy(void* dst, const void* src, size_t srcLen, size_t sliceLen) {
	gfmat_init();
	gf16_cksum_copy_generic(dst, src, srcLen, sliceLen);
}
int ref_cksum_copy_check(void* dst, const void* src, size_t len) {
	gfmat_init();
	return gf16_cksum_copy_check_generic(dst, src, len);
}

// Computes `numRec` recovery slices from `numIn` input slices through the
// reference CPU controller.  inputs: numIn rows of `sliceSize` bytes; row i
// holds lens[i] meaningful bytes (the rest is ignored, the controller
// zero-pads).  out: numRec rows of sliceSize bytes.  valid[r] = checksum
// verdict.  Returns 0 on success.
int ref_create(const uint8_t* inputs, const size_t* lens, const uint16_t* inputNums, unsigned numIn,
               size_t sliceSize, const uint16_t* exps, unsigned numRec,
               uint8_t* out, int* valid, int method, int threads, unsigned batch,
               double* seconds) {
	PAR2Proc proc;
	PAR2ProcCPU cpu(2);
	if(threads > 0) cpu.setNumThreads(threads);
	if(!proc.init(sliceSize, {{&cpu, 0, sliceSize}})) return -1;
	if(!cpu.init((Galois16Methods)method, batch)) return -2;
	g_method_name = cpu.getMethodName();
	if(!proc.setRecoverySlices(numRec, exps)) return -3;
	auto t0 = std::chrono::steady_clock::now();
	std::vector<std::future<void>> pending;
	for(unsigned i = 0; i < numIn; i++) {
		proc.waitForAdd();
		pending.push_back(proc.addInput(inputs + (size_t)i * sliceSize, lens[i], inputNums[i], false));
	}
	proc.endInput().get();
	for(auto& f : pending) f.get();
	auto t1 = std::chrono::steady_clock::now();
	if(seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
	for(unsigned r = 0; r < numRec; r++)
		valid[r] = proc.getOutput(r, out + (size_t)r * sliceSize).get() ? 1 : 0;
	proc.deinit();
	return 0;
}

// Same as ref_create but with explicit per-input coefficient columns
// (coeffs[i*numRec + r]), i.e. PAR2Proc::addInput(buf, size, coeffs, flush).
int ref_create_coeffs(const uint8_t* inputs, const size_t* lens, const uint16_t* coeffs, unsigned numIn,
                      size_t sliceSize, unsigned numRec, uint8_t* out, int* valid, int method) {
	PAR2Proc proc;
	PAR2ProcCPU cpu(2);
	if(!proc.init(sliceSize, {{&cpu, 0, sliceSize}})) return -1;
	if(!cpu.init((Galois16Methods)method, 0)) return -2;
	if(!proc.setRecoverySlices(numRec, nullptr)) return -3;
	std::vector<std::future<void>> pending;
	for(unsigned i = 0; i < numIn; i++) {
		proc.waitForAdd();
		pending.push_back(proc.addInput(inputs + (size_t)i * sliceSize, lens[i], coeffs + (size_t)i * numRec, false));
	}
	proc.endInput().get();
	for(auto& f : pending) f.get();
	for(unsigned r = 0; r < numRec; r++)
		valid[r] = proc.getOutput(r, out + (size_t)r * sliceSize).get() ? 1 : 0;
	proc.deinit();
	return 0;
}

const char* ref_last_method_name(void) { return g_method_name.c_str(); }

// Hashes one file the way the addon does (src/gf.cc:926-954, 1015-1039):
// per-slice MD5+CRC32 (20-byte IFSC entries, last slice zero-padded to
// sliceSize) and the file MD5.  The data is fed in `feed` byte pieces to
// exercise the streaming state.
void ref_hash_file(const uint8_t* data, size_t len, size_t sliceSize, size_t feed,
                   uint8_t* ifsc, uint8_t* fileMd5) {
	setup_hasher();
	IHasherInput* h = HasherInput_Create();
	size_t pos = 0, inSlice = 0;
	unsigned slice = 0;
	if(feed == 0) feed = len ? len : 1;
	while(pos < len) {
		size_t n = feed;
		if(n > len - pos) n = len - pos;
		if(n > sliceSize - inSlice) n = sliceSize - inSlice;
		h->update(data + pos, n);
		pos += n;
		inSlice += n;
		if(inSlice == sliceSize) {
			h->getBlock(ifsc + 20 * (slice++), 0);
			inSlice = 0;
		}
	}
	if(inSlice) h->getBlock(ifsc + 20 * (slice++), sliceSize - inSlice);
	h->end(fileMd5);
	h->destroy();
}

uint32_t ref_crc32(const void* data, size_t len) { setup_hasher(); return CRC32_Calc(data, len); }
uint32_t ref_md5crc(const void* data, size_t len, size_t zeroPad, void* md5) {
	setup_hasher();
	return MD5CRC_Calc(data, len, zeroPad, md5);
}

// MD5 of N equal-length buffers through MD5Multi (hasher/hasher.h:33-56),
// the recovery-packet hasher (src/gf.cc:1075-1219).
void ref_md5multi(const uint8_t* const* bufs, unsigned n, size_t len, uint8_t* md5s) {
	setup_hasher();
	MD5Multi m(n);
	m.update((const void* const*)bufs, len);
	m.end();
	m.get(md5s);
}

} // extern "C"
