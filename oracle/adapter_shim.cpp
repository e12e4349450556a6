// Test infrastructure only: drives the PAR2ProcCUDA adapter
// (parpar_gb300/adapter/controller_cuda.{h,cpp}) through the reference's own
// PAR2Proc (gf16/controller.cpp), alone or beside the reference's PAR2ProcCPU
// over split byte ranges of every slice (PAR2Proc::init with several backends,
// gf16/controller.cpp:13-130; the addon builds such lists in src/gf.cc:697-728),
// in chunked passes the way lib/par2.js PAR2Chunked drives GfProc
// (setCurrentSliceSize per window, discardOutput after each EndInput,
// src/gf.cc:439-460, 624-648).  Compiled by oracle/ref.mk into
// oracle/_ref/libparref_cuda.so; only tests/ load it.
#include "gf16/controller.h"
#include "gf16/controller_cpu.h"
#include "controller_cuda.h"

#include <algorithm>
#include <cstring>
#include <vector>

extern "C" {

// Recovery slices through PAR2Proc.
//   inputs: numIn rows `pitch` bytes apart, row i holding lens[i] bytes;
//   coeffs: NULL (PAR2 coefficients from inputNums/exps) or numIn x numRec
//           explicit columns (PAR2Proc::addInput(buf, size, coeffs));
//   cpuBytes: 0 = the CUDA backend alone, else PAR2ProcCPU takes bytes
//           [0, cpuBytes) of each slice and the CUDA backend the rest;
//   chunk: 0 = one pass, else passes over windows of `chunk` bytes;
//   out: numRec rows of sliceSize bytes; valid[r]: AND of the verdicts of
//   every pass; stats[0] = batches the CUDA backend started, stats[1] = its
//   input batch size.
// Returns 0, or negative: -1 PAR2Proc::init, -2 CUDA init, -3 CPU init,
// -4 setRecoverySlices, -5 setCurrentSliceSize.
int adapter_create(const uint8_t* inputs, size_t pitch, const size_t* lens, const uint16_t* inputNums,
                   const uint16_t* coeffs, unsigned numIn, size_t sliceSize, const uint16_t* exps, unsigned numRec,
                   uint8_t* out, int* valid, size_t cpuBytes, size_t chunk, int method, unsigned inputBatch,
                   unsigned* stats) {
	if(!chunk || chunk > sliceSize) chunk = sliceSize;
	PAR2Proc proc;
	PAR2ProcCUDA cuda(0, 2);
	PAR2ProcCPU cpu(2);
	std::vector<PAR2ProcBackendAlloc> alloc;
	if(cpuBytes && cpuBytes < chunk) {
		alloc.push_back({&cpu, 0, cpuBytes});
		alloc.push_back({&cuda, cpuBytes, chunk - cpuBytes});
	} else {
		alloc.push_back({&cuda, 0, chunk});
	}
	if(!proc.init(chunk, alloc)) return -1;
	if(!cuda.init(method, inputBatch)) return -2;
	if(alloc.size() > 1 && !cpu.init(GF16_AUTO, 0)) return -3;
	if(!proc.setRecoverySlices(numRec, exps)) return -4;
	std::vector<uint8_t> tmp(chunk);
	for(unsigned r = 0; r < numRec; r++) valid[r] = 1;
	size_t cur = chunk;
	for(size_t off = 0; off < sliceSize; off += chunk) {
		size_t len = std::min(chunk, sliceSize - off);
		if(off) proc.discardOutput();
		if(len != cur) {
			if(!proc.setCurrentSliceSize(len)) return -5;
			cur = len;
		}
		std::vector<std::future<void>> pending;
		pending.reserve(numIn);
		for(unsigned i = 0; i < numIn; i++) {
			size_t avail = lens[i] > off ? std::min(lens[i] - off, len) : 0;
			const uint8_t* src = inputs + (size_t)i * pitch + off;
			proc.waitForAdd();
			if(coeffs) pending.push_back(proc.addInput(src, avail, coeffs + (size_t)i * numRec, false));
			else pending.push_back(proc.addInput(src, avail, inputNums[i], false));
		}
		proc.endInput().get();
		for(auto& f : pending) f.get();
		for(unsigned r = 0; r < numRec; r++) {
			bool ok = proc.getOutput(r, tmp.data()).get();
			valid[r] = valid[r] && ok;
			memcpy(out + (size_t)r * sliceSize + off, tmp.data(), len);
		}
	}
	if(stats) {
		stats[0] = cuda.getBatchesStarted();
		stats[1] = cuda.getInputBatchSize();
	}
	proc.deinit();
	return 0;
}

// PAR2ProcCUDA on `device` with `stagingAreas`: 1 when init succeeds, 0 when
// it reports failure (no such device, bad argument), with the library's
// message copied into msg.
int adapter_probe(int device, int stagingAreas, char* msg, size_t msgLen) {
	PAR2ProcCUDA cuda(device, stagingAreas);
	cuda.setSliceSize(4096);
	bool ok = cuda.init();
	if(msg && msgLen) {
		strncpy(msg, ok ? "" : PAR2ProcCUDA::lastError(), msgLen - 1);
		msg[msgLen - 1] = 0;
	}
	return ok ? 1 : 0;
}

} // extern "C"
