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

#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>
#if defined(__aarch64__) && defined(__linux__)
#include <sys/auxv.h>
#endif

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

// One whole create job the way ParPar runs it on the CPU: the GF
// multiply-accumulate of every input into every recovery slice through
// PAR2Proc + PAR2ProcCPU (GF16_AUTO, `threads` workers, or the controller's
// own hardware_concurrency() default when threads <= 0,
// gf16/controller_cpu.cpp:52-55), and, concurrently, the input hashes of
// every file on a thread of its own, as each JS HasherInput object owns one
// (src/gf.cc:926-954, 1015-1039): per-slice MD5+CRC32 (IFSC, last slice
// zero-padded) and the file MD5.
//   inputs: numIn rows `pitch` bytes apart, row i holding lens[i] bytes;
//   file f: fileLens[f] bytes in the rows from firstRow[f];
//   out: numRec rows of sliceSize bytes; valid[r] the checksum verdicts;
//   ifsc: 20 bytes per row; fileMd5: 16 bytes per file;
//   times[0] = wall seconds of the whole job (both parts), times[1] = GF part
//   (first addInput to endInput completion), times[2] = hashing part.
int ref_job(const uint8_t* inputs, size_t pitch, const size_t* lens, const uint16_t* inputNums, unsigned numIn,
            size_t sliceSize, const uint16_t* exps, unsigned numRec, uint8_t* out, int* valid,
            const uint64_t* fileLens, const uint32_t* firstRow, unsigned numFiles, uint8_t* ifsc, uint8_t* fileMd5,
            int threads, double* times) {
	setup_hasher();
	PAR2Proc proc;
	PAR2ProcCPU cpu(2);
	if(threads > 0) cpu.setNumThreads(threads);
	if(!proc.init(sliceSize, {{&cpu, 0, sliceSize}})) return -1;
	if(!cpu.init(GF16_AUTO, 0)) return -2;
	g_method_name = cpu.getMethodName();
	if(!proc.setRecoverySlices(numRec, exps)) return -3;

	auto hashFile = [&](unsigned f) {
		IHasherInput* h = HasherInput_Create();
		uint64_t left = fileLens[f];
		size_t row = firstRow[f];
		uint8_t* entry = ifsc + 20 * row;
		while(left) {
			size_t n = left < sliceSize ? (size_t)left : sliceSize;
			h->update(inputs + row * pitch, n);
			h->getBlock(entry, sliceSize - n);
			entry += 20;
			row++;
			left -= n;
		}
		h->end(fileMd5 + 16 * f);
		h->destroy();
	};

	auto t0 = std::chrono::steady_clock::now();
	std::atomic<double> tHash(0.0);
	std::vector<std::thread> hashers;
	hashers.reserve(numFiles);
	std::atomic<unsigned> hashersLeft(numFiles);
	for(unsigned f = 0; f < numFiles; f++)
		hashers.emplace_back([&, f]() {
			hashFile(f);
			if(hashersLeft.fetch_sub(1) == 1)
				tHash = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
		});
	std::vector<std::future<void>> pending;
	pending.reserve(numIn);
	for(unsigned i = 0; i < numIn; i++) {
		proc.waitForAdd();
		pending.push_back(proc.addInput(inputs + (size_t)i * pitch, lens[i], inputNums[i], false));
	}
	proc.endInput().get();
	for(auto& f : pending) f.get();
	double tGf = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
	for(auto& t : hashers) t.join();
	double tAll = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
	for(unsigned r = 0; r < numRec; r++)
		valid[r] = proc.getOutput(r, out + (size_t)r * sliceSize).get() ? 1 : 0;
	proc.deinit();
	if(times) { times[0] = tAll; times[1] = tGf; times[2] = tHash; }
	return 0;
}

// The GF method GF16_AUTO resolves to on this host for `threads` workers,
// the worker count, and the CPU features the reference's dispatch reads
// (on aarch64: HWCAP ASIMD/PMULL/CRC32, HWCAP2 SVE2, HWCAP SVE), as text.
int ref_host_info(char* buf, size_t len) {
	PAR2ProcCPU cpu(1);
	cpu.setSliceSize(65536);
	if(!cpu.init(GF16_AUTO, 0)) return -1;
	std::string caps;
#if defined(__aarch64__) && defined(__linux__)
	unsigned long hw = getauxval(AT_HWCAP), hw2 = getauxval(AT_HWCAP2);
	char tmp[160];
	snprintf(tmp, sizeof(tmp), "hwcap=0x%lx hwcap2=0x%lx asimd=%d pmull=%d crc32=%d sve=%d sve2=%d", hw, hw2,
	         (int)((hw >> 1) & 1), (int)((hw >> 4) & 1), (int)((hw >> 7) & 1), (int)((hw >> 22) & 1), (int)((hw2 >> 1) & 1));
	caps = tmp;
#else
	caps = "x86";
#endif
	snprintf(buf, len, "method=%s;threads=%d;%s", cpu.getMethodName(), cpu.getNumThreads(), caps.c_str());
	cpu.deinit();
	return 0;
}

} // extern "C"
