// PAR2ProcCUDA: IPAR2ProcBackend over libpar2cuda (see controller_cuda.h).
#include "controller_cuda.h"

#include <cstdint>

struct PAR2ProcCUDA::Pending {
	PAR2ProcCUDA* self;
	int kind; // 0 = add, 1 = output, 2 = end
	int status;
#ifdef USE_LIBUV
	PAR2ProcPlainCb plainCb;
	PAR2ProcOutputCb outCb;
#else
	std::promise<void> done;
	std::promise<bool> valid;
#endif
};

// Runs on the library's notifier thread, in submission order per kind.
void PAR2ProcCUDA::doneCb(void* user, int status) {
	auto* p = static_cast<Pending*>(user);
	p->status = status;
#ifdef USE_LIBUV
	// hand over to the loop thread, as the OpenCL backend does
	if(p->kind == 1) p->self->_queueRecv.notify(p);
	else p->self->_queueSent.notify(p);
#else
	if(p->kind == 1) p->valid.set_value(status == 1);
	else p->done.set_value();
	delete p;
#endif
}

// One call per finished batch (the _notifyProc of the CPU backend,
// gf16/controller_cpu.cpp:627-645).
void PAR2ProcCUDA::progressTrampoline(void* user, unsigned numInputs) {
	auto* self = static_cast<PAR2ProcCUDA*>(user);
#ifdef USE_LIBUV
	self->_queueProc.notify(reinterpret_cast<void*>((uintptr_t)numInputs + 1));
#else
	(void)numInputs;
	self->stagingActiveCount_dec();
#endif
}

#ifdef USE_LIBUV
void PAR2ProcCUDA::_notifySent(void* req) {
	auto* p = static_cast<Pending*>(req);
	if(p->kind == 0) pendingInCallbacks--;
	if(p->plainCb) p->plainCb();
	delete p;
	if(endSignalled && isEmpty() && progressCb) progressCb(0);
}
void PAR2ProcCUDA::_notifyRecv(void* req) {
	auto* p = static_cast<Pending*>(req);
	pendingOutCallbacks--;
	p->outCb(p->status == 1);
	delete p;
	if(pendingOutCallbacks < 1 && deinitCallback) deinit(deinitCallback);
}
void PAR2ProcCUDA::_notifyProc(void* req) {
	stagingActiveCount_dec();
	if(progressCb) progressCb((unsigned)((uintptr_t)req - 1));
}
#endif

PAR2ProcCUDA::PAR2ProcCUDA(IF_LIBUV(uv_loop_t* loop,) int device, int stagingAreas)
: IPAR2ProcBackend(IF_LIBUV(loop)), ctx(nullptr), sliceSize(0) {
	ok = stagingAreas > 0 && par2cuda_create(device, (unsigned)stagingAreas, &ctx) == 0;
	processingAdd = false;
	statBatchesStarted = 0;
	currentStagingArea = currentStagingInputs = 0;
	inputBatchSize = minInBatchSize = 0;
	if(ok) par2cuda_set_progress_cb(ctx, &PAR2ProcCUDA::progressTrampoline, this);
}
PAR2ProcCUDA::~PAR2ProcCUDA() { deinit(); }
void PAR2ProcCUDA::_deinit() {
	if(ctx) {
		par2cuda_sync(ctx);
		par2cuda_destroy(ctx);
	}
	ctx = nullptr;
}

void PAR2ProcCUDA::setSliceSize(size_t size) {
	sliceSize = size;
	if(ctx) par2cuda_set_slice_size(ctx, size);
}
bool PAR2ProcCUDA::init(int method, unsigned inputBatch) {
	if(!ok || par2cuda_init(ctx, method, inputBatch) < 0) return false;
	par2cuda_info inf;
	if(par2cuda_info_get(ctx, &inf) < 0) return false;
	inputBatchSize = inf.staging_size;
	minInBatchSize = inf.min_staging_size;
	return true;
}
bool PAR2ProcCUDA::setCurrentSliceSize(size_t size) {
	return ctx && par2cuda_set_current_slice_size(ctx, size) == 0;
}
bool PAR2ProcCUDA::setRecoverySlices(unsigned n, const uint16_t* exps) {
	// explicit-coefficient use passes no exponents; the count still matters
	// (IPAR2ProcBackend::getNumRecoverySlices)
	if(exps) outputExponents.assign(exps, exps + n);
	else outputExponents.assign(n, 0);
	return ctx && par2cuda_set_recovery_slices(ctx, n, exps) == 0;
}
PAR2ProcBackendAddResult PAR2ProcCUDA::canAdd() const {
	int r = ctx ? par2cuda_can_add(ctx) : -1;
	return r == PAR2CUDA_ADD_OK ? PROC_ADD_OK : r == PAR2CUDA_ADD_OK_BUSY ? PROC_ADD_OK_BUSY : PROC_ADD_FULL;
}
// a return of 1 from an add / flush / dummy call means the call submitted a
// batch: the controller-visible active count goes up until its progress call
void PAR2ProcCUDA::noteSubmit(int rc) {
	if(rc == 1) {
		stagingActiveCount_inc();
		statBatchesStarted++;
	}
}
// discardOutput() is a base-class inline that only clears processingAdd; the
// first add after it tells the library to overwrite the recovery rows
void PAR2ProcCUDA::beginAdd() {
	if(!processingAdd) par2cuda_discard_output(ctx);
	processingAdd = true;
}

FUTURE_RETURN_T PAR2ProcCUDA::addInput(const void* buffer, size_t size, uint16_t inputNum, bool flush IF_LIBUV(, const PAR2ProcPlainCb& cb)) {
	beginAdd();
	auto* p = new Pending{this, 0, 0};
#ifdef USE_LIBUV
	p->plainCb = cb;
	pendingInCallbacks++;
#else
	auto fut = p->done.get_future();
#endif
	int rc = par2cuda_add_input(ctx, buffer, size, inputNum, flush, &PAR2ProcCUDA::doneCb, p);
	if(rc < 0) doneCb(p, rc); // the request never reached the library: complete it here
	else noteSubmit(rc);
	IF_NOT_LIBUV(return fut);
}
FUTURE_RETURN_T PAR2ProcCUDA::addInput(const void* buffer, size_t size, const uint16_t* coeffs, bool flush IF_LIBUV(, const PAR2ProcPlainCb& cb)) {
	beginAdd();
	auto* p = new Pending{this, 0, 0};
#ifdef USE_LIBUV
	p->plainCb = cb;
	pendingInCallbacks++;
#else
	auto fut = p->done.get_future();
#endif
	int rc = par2cuda_add_input_coeffs(ctx, buffer, size, coeffs, flush, &PAR2ProcCUDA::doneCb, p);
	if(rc < 0) doneCb(p, rc);
	else noteSubmit(rc);
	IF_NOT_LIBUV(return fut);
}
void PAR2ProcCUDA::dummyInput(uint16_t inputNum, bool flush) {
	beginAdd();
	noteSubmit(par2cuda_dummy_input(ctx, inputNum, flush));
}
bool PAR2ProcCUDA::fillInput(const void* buffer) { return par2cuda_fill_input(ctx, buffer) == 1; }
void PAR2ProcCUDA::flush() { noteSubmit(par2cuda_flush(ctx)); }

#ifndef USE_LIBUV
void PAR2ProcCUDA::waitForAdd() { par2cuda_wait_for_add(ctx); }
FUTURE_RETURN_T PAR2ProcCUDA::endInput() {
	auto* p = new Pending{this, 2, 0};
	auto fut = p->done.get_future();
	noteSubmit(par2cuda_flush(ctx));
	if(par2cuda_end_input(ctx, &PAR2ProcCUDA::doneCb, p) < 0) doneCb(p, -1);
	return fut;
}
#endif

FUTURE_RETURN_BOOL_T PAR2ProcCUDA::getOutput(unsigned index, void* output IF_LIBUV(, const PAR2ProcOutputCb& cb)) {
	auto* p = new Pending{this, 1, 0};
#ifdef USE_LIBUV
	p->outCb = cb;
	pendingOutCallbacks++;
#else
	auto fut = p->valid.get_future();
#endif
	// a failed call reports the slice as invalid (the reference's only error
	// channel on this path is the checksum verdict)
	if(par2cuda_get_output(ctx, index, output, &PAR2ProcCUDA::doneCb, p) < 0) doneCb(p, -1);
	IF_NOT_LIBUV(return fut);
}
void PAR2ProcCUDA::freeProcessingMem() {
	if(ctx) par2cuda_free_processing_mem(ctx);
}
bool PAR2ProcCUDA::info(par2cuda_info* out) const { return ctx && par2cuda_info_get(ctx, out) == 0; }
