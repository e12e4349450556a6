// PAR2ProcCUDA — ParPar's backend plugin interface (IPAR2ProcBackend,
// gf16/controller.h:77-217) over the par2cuda C ABI (include/par2cuda.h).
//
// In a ParPar tree this pair of files is gf16/controller_cuda.{h,cpp}; it
// compiles against the reference's own gf16/controller.h in both of its
// threading modes:
//   - without USE_LIBUV (the C++ std::future API used by PAR2Proc's callers
//     outside node), completions resolve futures;
//   - with USE_LIBUV (the node addon, src/gf.cc), the library's completion
//     callbacks are re-posted to the loop thread through the base class's
//     ThreadNotifyQueues (_queueSent / _queueRecv / _queueProc), the way the
//     OpenCL backend hands its completions over (gf16/controller_ocl.cpp:485-494).
// The controller-visible state that the base class keeps inline
// (processingAdd, stagingActiveCount, pendingIn/OutCallbacks,
// statBatchesStarted, inputBatchSize, minInBatchSize) is maintained here:
// par2cuda_add_input, par2cuda_flush and par2cuda_dummy_input return 1 when
// the call submitted a batch, and the library's progress callback fires once
// per finished batch.
#ifndef __GF16_CONTROLLER_CUDA
#define __GF16_CONTROLLER_CUDA

#include "controller.h"
#include "par2cuda.h"

class PAR2ProcCUDA : public IPAR2ProcBackend {
	par2cuda_ctx* ctx;
	size_t sliceSize;
	bool ok;
	struct Pending; // one per add / output / end request in flight
	static void doneCb(void* user, int status);
	static void progressTrampoline(void* user, unsigned numInputs);
	// batches are submitted inside the library (its transfer thread), so the
	// base class's kernel hook is never called
	void run_kernel(unsigned, unsigned) override {}
#ifdef USE_LIBUV
	void _notifySent(void* req) override;
	void _notifyRecv(void* req) override;
	void _notifyProc(void* req) override;
#endif
	void _deinit() override;
	void noteSubmit(int rc);
	void beginAdd();

	PAR2ProcCUDA(const PAR2ProcCUDA&);
	PAR2ProcCUDA& operator=(const PAR2ProcCUDA&);
public:
	// PAR2ProcOCL(loop, platformId, deviceId, stagingAreas) counterpart
	// (gf16/controller_ocl.h:188); stagingAreas as src/gf.cc:326-330 parses it
	explicit PAR2ProcCUDA(IF_LIBUV(uv_loop_t* loop,) int device = 0, int stagingAreas = 2);
	~PAR2ProcCUDA();
	// init(method, inputBatch): false ("Failed to allocate memory" in the addon)
	// when the device is missing or the library could not allocate
	bool init(int method = PAR2CUDA_METHOD_AUTO, unsigned inputBatch = 0);
	void setSliceSize(size_t size) override;
	bool setCurrentSliceSize(size_t size) override;
	bool setRecoverySlices(unsigned numSlices, const uint16_t* exponents = nullptr) override;
	PAR2ProcBackendAddResult canAdd() const override;
	FUTURE_RETURN_T addInput(const void* buffer, size_t size, uint16_t inputNum, bool flush IF_LIBUV(, const PAR2ProcPlainCb& cb)) override;
	FUTURE_RETURN_T addInput(const void* buffer, size_t size, const uint16_t* coeffs, bool flush IF_LIBUV(, const PAR2ProcPlainCb& cb)) override;
	void dummyInput(uint16_t inputNum, bool flush = false) override;
	bool fillInput(const void* buffer) override;
	void flush() override;
#ifndef USE_LIBUV
	FUTURE_RETURN_T endInput() override;
	void waitForAdd() override;
#endif
	FUTURE_RETURN_BOOL_T getOutput(unsigned index, void* output IF_LIBUV(, const PAR2ProcOutputCb& cb)) override;
	void processing_finished() override {}
	void freeProcessingMem() override;
	// GfProc.info() fields (src/gf.cc:527-568)
	bool info(par2cuda_info* out) const;
	// the library's message for the last failed call on this thread
	static const char* lastError() { return par2cuda_last_error(); }
};

#endif
