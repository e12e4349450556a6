// PAR2ProcCUDA: the backend object behind par2cuda_* (include/par2cuda.h).
//
// It keeps the observable behaviour of ParPar's backends
// (IPAR2ProcBackend, gf16/controller.h:77-217), following the OpenCL
// backend's structure (gf16/controller_ocl.cpp):
//   - `stagingAreas` input batches of `inputBatchSize` slots each; canAdd /
//     waitForAdd back-pressure on the current area (controller_ocl.cpp:265-273);
//   - the submit rule of _addInput (flush || batch full || idle and >= the
//     minimum batch, controller_ocl.cpp:329-343);
//   - processingAdd: the first batch after a discard overwrites the recovery
//     rows, later ones accumulate (controller_ocl.cpp:504-512);
//   - one transfer thread that performs copies and submits batches, and
//     notification of completions from a second thread
//     (controller_ocl.cpp:275-300, 485-494).
// The device side replaces the OpenCL buffers: the staged rows live in HBM,
// copies go on a copy stream, batches on a compute stream ordered after their
// copies with events, and completion is observed by cudaEventSynchronize on
// the notifier thread.
#include "engine.h"

#include <cstdio>
#include <cstring>

namespace p2c {

const uint16_t* host_input_logs();

static size_t default_batch(size_t slice, int method) {
	// about 512 MiB of staged input per area, 8..512 inputs, multiple of 8;
	// the 4-bit tensor method wants long K (16 bits per input) per GEMM: its
	// per-tile set-up and epilogue are amortised over more MMAs, so 4 GiB per
	// area, up to 4096 inputs (2000 x 2 MiB slices: 65 ms per pass through the
	// plugin calls against 96 ms with 256-input batches)
	const bool tensor4 = method == 5;
	size_t b = ((tensor4 ? 4096ull : 512ull) << 20) / (slice ? slice : 1);
	b = std::min<size_t>(b, tensor4 ? 4096 : 512);
	if(b < 8) b = 8;
	return round_up(b, 8);
}

Engine::Engine(int dev, unsigned areas) : device(dev), staging(areas ? areas : 1) {}

Engine::~Engine() { shutdown(); }

int Engine::start() {
	P2C_CUDA_TRY(cudaSetDevice(device));
	if(gf_tables(device, &gt)) return -1;
	P2C_CUDA_TRY(cudaStreamCreateWithFlags(&sCopy, cudaStreamNonBlocking));
	P2C_CUDA_TRY(cudaStreamCreateWithFlags(&sCompute, cudaStreamNonBlocking));
	P2C_CUDA_TRY(cudaStreamCreateWithFlags(&sOut, cudaStreamNonBlocking));
	running = true;
	transferThread = std::thread([this] { transfer_loop(); });
	notifyThread = std::thread([this] { notify_loop(); });
	return 0;
}

void Engine::shutdown() {
	if(running) {
		{
			std::lock_guard<std::mutex> lk(qm);
			tq.push_back(Req{Req::STOP});
		}
		qcv.notify_all();
		transferThread.join();
		{
			std::lock_guard<std::mutex> lk(nm);
			nq.push_back(Note{nullptr, {}, true});
		}
		ncv.notify_all();
		notifyThread.join();
		running = false;
	}
	cudaSetDevice(device);
	if(sCompute) cudaStreamSynchronize(sCompute);
	free_staging();
	free_processing();
	for(cudaEvent_t e : eventPool) cudaEventDestroy(e);
	eventPool.clear();
	if(sCopy) cudaStreamDestroy(sCopy);
	if(sCompute) cudaStreamDestroy(sCompute);
	if(sOut) cudaStreamDestroy(sOut);
	sCopy = sCompute = sOut = nullptr;
	if(hOutBounce) cudaFreeHost(hOutBounce);
	hOutBounce = nullptr;
}

// ------------------------------------------------------------------ memory
void Engine::free_staging() {
	for(auto& a : staging) {
		if(a.dIn) cudaFree(a.dIn);
		if(a.hBounce) cudaFreeHost(a.hBounce);
		if(a.hDesc) cudaFreeHost(a.hDesc);
		if(a.dDesc) cudaFree(a.dDesc);
		a.dIn = nullptr; a.hBounce = nullptr; a.hDesc = nullptr; a.dDesc = nullptr;
		a.bounceBytes = 0;
		a.descBytes = 0;
	}
	stagingPitch = 0;
}

void Engine::free_processing() {
	if(dRec) cudaFree(dRec);
	if(dScratch) cudaFree(dScratch);
	if(hFlags) cudaFreeHost(hFlags);
	dRec = nullptr; dScratch = nullptr; hFlags = nullptr;
	recRowsAlloc = 0; recPitchAlloc = 0; scratchBytes = 0;
}

size_t Engine::desc_bytes() const {
	// lens u32[Bpad] | logs u16[Bpad] | custom u16[Bpad][R] | outExp u16[R]
	size_t R = outputExponents.size() ? outputExponents.size() : 1;
	return round_up((size_t)batchPad * 4, 16) + round_up((size_t)batchPad * 2, 16) +
	       round_up((size_t)batchPad * R * 2, 16) + round_up(R * 2, 16);
}

int Engine::alloc_staging() {
	P2C_CUDA_TRY(cudaSetDevice(device));
	size_t pitch = row_pitch(allocSliceSize);
	if(pitch != stagingPitch) {
		for(auto& a : staging) {
			if(a.dIn) cudaFree(a.dIn);
			a.dIn = nullptr;
			P2C_CUDA_TRY(cudaMalloc(&a.dIn, (size_t)batchPad * pitch * 2));
			// zero once so that table-build reads of unused slots are defined
			P2C_CUDA_TRY(cudaMemset(a.dIn, 0, (size_t)batchPad * pitch * 2));
		}
		stagingPitch = pitch;
	}
	return alloc_desc();
}

int Engine::alloc_desc() {
	size_t need = desc_bytes();
	for(auto& a : staging) {
		if(a.descBytes < need) {
			if(a.hDesc) cudaFreeHost(a.hDesc);
			if(a.dDesc) cudaFree(a.dDesc);
			a.hDesc = nullptr; a.dDesc = nullptr;
			P2C_CUDA_TRY(cudaHostAlloc(&a.hDesc, need, cudaHostAllocDefault));
			P2C_CUDA_TRY(cudaMalloc(&a.dDesc, need));
			a.descBytes = need;
		}
		a.logs.assign(batchPad, 0);
		a.lens.assign(batchPad, 0);
		a.custom.assign((size_t)batchPad * std::max<size_t>(1, outputExponents.size()), 0);
		a.hasCustom = false;
	}
	return 0;
}

size_t Engine::fp4_scratch_bytes() const {
	// the coefficient bit matrix of a full batch plus word chunks of at most
	// 512 MiB of expanded input planes
	return tc4_scratch_chunked_bytes((unsigned)outputExponents.size(), batchPad, row_words(allocSliceSize), 512ull << 20);
}

int Engine::alloc_processing() {
	P2C_CUDA_TRY(cudaSetDevice(device));
	size_t R = outputExponents.size();
	size_t pitch = row_pitch(allocSliceSize);
	if(R > recRowsAlloc || pitch != recPitchAlloc) {
		if(dRec) cudaFree(dRec);
		dRec = nullptr;
		P2C_CUDA_TRY(cudaMalloc(&dRec, R * pitch * 2));
		recRowsAlloc = R;
		recPitchAlloc = pitch;
		processingAdd = false;
		if(hFlags) cudaFreeHost(hFlags);
		hFlags = nullptr;
		P2C_CUDA_TRY(cudaHostAlloc(&hFlags, R ? R : 1, cudaHostAllocDefault));
	}
	// scratch: index bytes + coefficient matrix + checksum accumulators + flags
	size_t need = round_up(std::max(idx_bytes((unsigned)R, batchPad), tc_scratch_bytes((unsigned)R, batchPad)), 256) +
	              round_up(R * batchPad * 2, 256) +
	              round_up(std::max<size_t>(R, batchPad) * 8, 256) + round_up(R, 256);
	// the 4-bit tensor method's operand planes follow (method 5 only)
	if(method == 5) need += fp4_scratch_bytes();
	if(need > scratchBytes) {
		if(dScratch) cudaFree(dScratch);
		dScratch = nullptr;
		P2C_CUDA_TRY(cudaMalloc(&dScratch, need));
		scratchBytes = need;
	}
	return 0;
}

// ------------------------------------------------------------------ config
int Engine::init(int m, unsigned inputBatch) {
	if(!sliceSize) { set_error("setSliceSize must be called before init"); return -1; }
	method = m == 0 ? 1 : m;
	if(method < 1 || method > 5) { set_error("unknown method %d", m); return -1; }
	inputBatchSize = inputBatch ? inputBatch : (unsigned)default_batch(sliceSize, method);
	if(inputBatchSize > 32768) { set_error("input batch size %u > 32768", inputBatchSize); return -1; }
	batchPad = (unsigned)round_up(inputBatchSize, 8);
	minInBatchSize = inputBatchSize;
	allocSliceSize = std::max(allocSliceSize, sliceSize);
	currentSliceSize = sliceSize;
	currentStagingArea = currentStagingInputs = 0;
	statBatchesStarted = 0;
	stagingActiveCount = 0;
	processingAdd = false;
	for(auto& a : staging) a.active = false;
	initialised = true;
	if(alloc_staging()) {
		// leave nothing half-allocated: the backend refuses inputs until a
		// later init succeeds
		free_staging();
		initialised = false;
		return -1;
	}
	// a new method or batch size changes the scratch that recovery rows
	// already set need
	if(!outputExponents.empty() && alloc_processing()) {
		free_processing();
		outputExponents.clear();
		return -1;
	}
	return 0;
}

int Engine::set_slice_size(size_t s) {
	if(s < 2 || (s & 1)) { set_error("slice size %zu must be even and >= 2", s); return -1; }
	sliceSize = s;
	return 0;
}

int Engine::set_current_slice_size(size_t s) {
	// 0: PAR2Proc gives this backend no bytes of a short last window when it
	// splits slices over several backends (gf16/controller.cpp:100-112); it
	// then adds nothing to it, and the CPU backend accepts the size as well
	if(s && (s < 2 || (s & 1))) { set_error("slice size %zu must be even and >= 2", s); return -1; }
	wait_idle();
	currentSliceSize = s;
	if(s > allocSliceSize) {
		// upsizing: reallocate (PAR2ProcCPU::setCurrentSliceSize, controller_cpu.cpp:147-168)
		allocSliceSize = s;
		sliceSize = std::max(sliceSize, s);
		if(initialised && alloc_staging()) {
			free_staging();
			initialised = false;
			return -1;
		}
		if(!outputExponents.empty() && alloc_processing()) {
			free_processing();
			outputExponents.clear();
			return -1;
		}
	}
	return 0;
}

int Engine::set_recovery_slices(unsigned n, const uint16_t* exps) {
	wait_idle();
	outputExponents.assign(n, 1); // 1 when only explicit coefficients are used (controller_cpu.cpp:176)
	if(exps) for(unsigned i = 0; i < n; i++) outputExponents[i] = exps[i];
	if(!n) return 0;
	if(!initialised) { set_error("init must be called before setRecoverySlices"); return -1; }
	if(alloc_desc() || alloc_processing()) {
		// the reference reports this as "Failed to allocate memory"; the
		// backend then holds no recovery rows and refuses inputs until a
		// later setRecoverySlices succeeds
		free_processing();
		outputExponents.clear();
		return -1;
	}
	return 0;
}

// ------------------------------------------------------------------ adding
int Engine::can_add() const {
	if(staging[currentStagingArea].active) return 2; // FULL
	return stagingActiveCount.load() < staging.size() - 1 ? 0 : 1;
}

int Engine::wait_for_add() {
	Area& a = staging[currentStagingArea];
	std::unique_lock<std::mutex> lk(a.m);
	a.cv.wait(lk, [&] { return !a.active.load(); });
	return 0;
}

int Engine::add_input(const void* buf, size_t size, int inputNum, const uint16_t* coeffs, bool flush,
                      par2cuda_done_fn cb, void* user, bool dummy) {
	if(!initialised || outputExponents.empty()) { set_error("setRecoverySlices not yet called"); return -1; }
	if(size > currentSliceSize) { set_error("input of %zu bytes exceeds the slice size %zu", size, currentSliceSize); return -1; }
	if(!coeffs && (inputNum < 0 || inputNum > 32767)) { set_error("input index %d not valid", inputNum); return -1; }
	Area& a = staging[currentStagingArea];
	if(a.active) { set_error("staging area busy (canAdd() is FULL)"); return -1; }
	const unsigned slot = currentStagingInputs;
	// set_coeffs (controller_ocl.cpp:387-403); PAR2 rows of a batch that also
	// holds explicit coefficients are expanded on the host in run_kernel
	const size_t R = outputExponents.size();
	if(coeffs) {
		memcpy(&a.custom[(size_t)slot * R], coeffs, R * 2);
		a.hasCustom = true;
		a.logs[slot] = 0;
	} else {
		a.logs[slot] = host_input_logs()[inputNum];
	}
	a.lens[slot] = dummy ? (uint32_t)currentSliceSize : (uint32_t)size;
	currentStagingInputs++;
	unsigned submit = (flush || currentStagingInputs == inputBatchSize ||
	                   (stagingActiveCount.load() == 0 && staging.size() > 1 && currentStagingInputs >= minInBatchSize))
	                  ? currentStagingInputs : 0;
	Req rq{dummy ? Req::DUMMY : Req::ADD};
	rq.buf = buf; rq.size = size; rq.area = currentStagingArea; rq.slot = slot;
	rq.submit = submit; rq.cb = cb; rq.user = user;
	if(submit) {
		stagingActiveCount++;
		a.active = true;
		statBatchesStarted++;
		currentStagingInputs = 0;
		if(++currentStagingArea == staging.size()) currentStagingArea = 0;
	}
	enqueue(rq);
	return submit ? 1 : 0;
}

int Engine::fill_input(const void* buf) {
	if(!initialised) { set_error("init not called"); return -1; }
	Req rq{Req::FILL};
	rq.buf = buf; rq.size = currentSliceSize; rq.area = currentStagingArea; rq.slot = currentStagingInputs;
	staging[currentStagingArea].lens[currentStagingInputs] = (uint32_t)currentSliceSize;
	enqueue(rq);
	if(++currentStagingInputs == inputBatchSize) {
		currentStagingInputs = 0;
		if(++currentStagingArea == staging.size()) {
			currentStagingArea = 0;
			return 1;
		}
	}
	return 0;
}

int Engine::flush() {
	if(!currentStagingInputs) return 0;
	Req rq{Req::FLUSH};
	rq.area = currentStagingArea;
	rq.submit = currentStagingInputs;
	stagingActiveCount++;
	staging[currentStagingArea].active = true;
	statBatchesStarted++;
	currentStagingInputs = 0;
	if(++currentStagingArea == staging.size()) currentStagingArea = 0;
	enqueue(rq);
	return 1;
}

int Engine::end_input(par2cuda_done_fn cb, void* user) {
	if(flush() < 0) return -1;
	Req rq{Req::END};
	rq.cb = cb; rq.user = user;
	enqueue(rq);
	return 0;
}

int Engine::get_output(unsigned index, void* out, par2cuda_done_fn cb, void* user) {
	if(index >= outputExponents.size()) { set_error("recovery index %u not valid", index); return -1; }
	Req rq{Req::OUTPUT};
	rq.buf = out; rq.slot = index; rq.cb = cb; rq.user = user;
	enqueue(rq);
	return 0;
}

int Engine::output_valid(unsigned index) {
	if(index >= outputExponents.size()) { set_error("recovery index %u not valid", index); return -1; }
	sync();
	if(!processingAdd) return 1;   // nothing computed: zeros, valid
	return hFlags ? (int)hFlags[index] : -1;
}

int Engine::sync() {
	std::unique_lock<std::mutex> lk(qm);
	idleCv.wait(lk, [&] { return tq.empty() && !transferBusy; });
	lk.unlock();
	std::unique_lock<std::mutex> nl(nm);
	nIdleCv.wait(nl, [&] { return nq.empty() && !notifyBusy; });
	return lastAsyncError;
}

void Engine::wait_idle() {
	if(running) sync();
}

int Engine::free_processing_mem() {
	wait_idle();
	free_processing();
	processingAdd = false;
	return 0;
}

uint16_t Engine::host_exp(uint32_t e) {
	static uint16_t tab[65535];
	static std::once_flag once;
	std::call_once(once, [] {
		uint32_t n = 1;
		for(uint32_t i = 0; i < 65535; i++) { tab[i] = (uint16_t)n; n <<= 1; if(n & 0x10000) n ^= P2C_POLY; }
	});
	return tab[e % 65535];
}

// ------------------------------------------------------------------ threads
void Engine::enqueue(const Req& r) {
	{
		std::lock_guard<std::mutex> lk(qm);
		tq.push_back(r);
	}
	qcv.notify_one();
}

void Engine::notify_after(cudaStream_t st, std::function<void()> fn) {
	cudaEvent_t ev = take_event();
	cudaEventRecord(ev, st);
	{
		std::lock_guard<std::mutex> lk(nm);
		nq.push_back(Note{ev, std::move(fn), false});
	}
	ncv.notify_one();
}

cudaEvent_t Engine::take_event() {
	std::lock_guard<std::mutex> lk(em);
	if(!eventPool.empty()) {
		cudaEvent_t e = eventPool.back();
		eventPool.pop_back();
		return e;
	}
	cudaEvent_t e = nullptr;
	cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
	return e;
}

void Engine::give_event(cudaEvent_t e) {
	std::lock_guard<std::mutex> lk(em);
	eventPool.push_back(e);
}

void Engine::notify_loop() {
	cudaSetDevice(device);
	for(;;) {
		Note n;
		{
			std::unique_lock<std::mutex> lk(nm);
			ncv.wait(lk, [&] { return !nq.empty(); });
			n = std::move(nq.front());
			nq.pop_front();
			notifyBusy = true;
		}
		if(n.stop) {
			std::lock_guard<std::mutex> lk(nm);
			notifyBusy = false;
			nIdleCv.notify_all();
			return;
		}
		cudaError_t e = cudaEventSynchronize(n.ev);
		if(e != cudaSuccess) {
			set_error("device error: %s", cudaGetErrorString(e));
			lastAsyncError = -1;
		}
		give_event(n.ev);
		if(n.fn) n.fn();
		{
			std::lock_guard<std::mutex> lk(nm);
			notifyBusy = false;
			if(nq.empty()) nIdleCv.notify_all();
		}
	}
}

static bool is_pinned(const void* p) {
	cudaPointerAttributes at;
	if(cudaPointerGetAttributes(&at, p) != cudaSuccess) { cudaGetLastError(); return false; }
	return at.type == cudaMemoryTypeHost || at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

void Engine::transfer_loop() {
	cudaSetDevice(device);
	for(;;) {
		Req r;
		{
			std::unique_lock<std::mutex> lk(qm);
			qcv.wait(lk, [&] { return !tq.empty(); });
			r = tq.front();
			tq.pop_front();
			transferBusy = true;
		}
		if(r.kind == Req::STOP) {
			std::lock_guard<std::mutex> lk(qm);
			transferBusy = false;
			idleCv.notify_all();
			return;
		}
		int rc = 0;
		switch(r.kind) {
		case Req::ADD: case Req::FILL: rc = do_copy(r); break;
		case Req::DUMMY: if(r.submit) rc = run_kernel(r.area, r.submit); break;
		case Req::FLUSH: rc = run_kernel(r.area, r.submit); break;
		case Req::END: rc = do_end(r); break;
		case Req::OUTPUT: rc = do_output(r); break;
		default: break;
		}
		if(rc) {
			lastAsyncError = -1;
			fprintf(stderr, "par2cuda: %s\n", get_error());
		}
		{
			std::lock_guard<std::mutex> lk(qm);
			transferBusy = false;
			if(tq.empty()) idleCv.notify_all();
		}
	}
}

int Engine::do_copy(const Req& r) {
	Area& a = staging[r.area];
	uint16_t* dRow = a.dIn + (size_t)r.slot * stagingPitch;
	if(r.size) {
		if(is_pinned(r.buf)) {
			P2C_CUDA_TRY(cudaMemcpyAsync(dRow, r.buf, r.size, cudaMemcpyDefault, sCopy));
		} else {
			size_t need = (size_t)batchPad * allocSliceSize;
			if(a.bounceBytes < need) {
				if(a.hBounce) { cudaStreamSynchronize(sCopy); cudaFreeHost(a.hBounce); }
				a.hBounce = nullptr;
				P2C_CUDA_TRY(cudaHostAlloc(&a.hBounce, need, cudaHostAllocDefault));
				a.bounceBytes = need;
			}
			uint8_t* hb = a.hBounce + (size_t)r.slot * allocSliceSize;
			memcpy(hb, r.buf, r.size);
			P2C_CUDA_TRY(cudaMemcpyAsync(dRow, hb, r.size, cudaMemcpyHostToDevice, sCopy));
		}
	}
	if(r.kind == Req::ADD) {
		par2cuda_done_fn cb = r.cb;
		void* user = r.user;
		// the source buffer is free once the copy has run
		notify_after(sCopy, [cb, user] { if(cb) cb(user, 0); });
	}
	if(r.submit) return run_kernel(r.area, r.submit);
	return 0;
}

// one batch: descriptors, zero padding + checksum, coefficients, multiply-accumulate
int Engine::run_kernel(unsigned areaIdx, unsigned numInputs) {
	Area& a = staging[areaIdx];
	const unsigned R = (unsigned)outputExponents.size();
	const size_t pitch = stagingPitch;
	const size_t S = currentSliceSize;
	if(!R) { finish_area(areaIdx, numInputs); return 0; }
	// ordered after this batch's copies
	cudaEvent_t ev = take_event();
	P2C_CUDA_TRY(cudaEventRecord(ev, sCopy));
	P2C_CUDA_TRY(cudaStreamWaitEvent(sCompute, ev, 0));
	give_event(ev); // safe: the wait has captured the event's state

	// descriptor block (pinned -> device)
	uint8_t* h = a.hDesc;
	const size_t oLens = 0, oLogs = round_up((size_t)batchPad * 4, 16);
	const size_t oCustom = oLogs + round_up((size_t)batchPad * 2, 16);
	const size_t oExp = oCustom + round_up((size_t)batchPad * R * 2, 16);
	// the previous use of this area's descriptors has finished (area was inactive)
	memcpy(h + oLens, a.lens.data(), numInputs * 4);
	memcpy(h + oLogs, a.logs.data(), numInputs * 2);
	const bool custom = a.hasCustom;
	if(custom) {
		// rows of PAR2 inputs in a mixed batch get their coefficients here
		for(unsigned s = 0; s < numInputs; s++) {
			if(a.logs[s]) for(unsigned rr = 0; rr < R; rr++)
				a.custom[(size_t)s * R + rr] = host_exp(((uint32_t)a.logs[s] * outputExponents[rr]) % 65535u);
		}
		memcpy(h + oCustom, a.custom.data(), (size_t)numInputs * R * 2);
	}
	memcpy(h + oExp, outputExponents.data(), (size_t)R * 2);
	size_t copyBytes = oExp + (size_t)R * 2;
	P2C_CUDA_TRY(cudaMemcpyAsync(a.dDesc, h, copyBytes, cudaMemcpyHostToDevice, sCompute));
	const uint32_t* dLens = reinterpret_cast<const uint32_t*>(a.dDesc + oLens);
	const uint16_t* dLogs = reinterpret_cast<const uint16_t*>(a.dDesc + oLogs);
	const uint16_t* dCustom = custom ? reinterpret_cast<const uint16_t*>(a.dDesc + oCustom) : nullptr;
	const uint16_t* dExp = reinterpret_cast<const uint16_t*>(a.dDesc + oExp);

	// scratch carve-up
	uint8_t* sp = reinterpret_cast<uint8_t*>(dScratch);
	uint4* dIdx = reinterpret_cast<uint4*>(sp);
	sp += round_up(std::max(idx_bytes(R, batchPad), tc_scratch_bytes(R, batchPad)), 256);
	uint16_t* dCoeff = reinterpret_cast<uint16_t*>(sp);
	sp += round_up((size_t)R * batchPad * 2, 256);
	unsigned long long* dCk = reinterpret_cast<unsigned long long*>(sp);

	if(rows_cksum(a.dIn, pitch, numInputs, dLens, S, dCk, 0, nullptr, gt, sCompute)) return -1;
	const bool needCoeff = method != 1;
	if(make_idx(dLogs, dCustom, dExp, R, numInputs, dIdx, needCoeff ? dCoeff : nullptr, gt, sCompute)) return -1;
	const size_t nWords = row_words(S);
	const int acc = processingAdd ? 1 : 0;
	int rc = 0;
	if(method == 2) rc = xor_planes_muladd(a.dIn, pitch, numInputs, dCoeff, dRec, recPitchAlloc, R, nWords, acc, sCompute);
	else if(method == 3) rc = nibble_muladd_t(a.dIn, pitch, numInputs, dCoeff, dRec, recPitchAlloc, R, nWords, acc, gt, sCompute);
	else if(method == 4) rc = tc_muladd(a.dIn, pitch, numInputs, dCoeff, dRec, recPitchAlloc, R, nWords, acc, true, dIdx,
	                                    tc_scratch_bytes(R, numInputs), sCompute);
	else if(method == 5) {
		uint8_t* fp = reinterpret_cast<uint8_t*>(dScratch) + (scratchBytes - fp4_scratch_bytes());
		rc = tc4_muladd(a.dIn, pitch, numInputs, dCoeff, dRec, recPitchAlloc, R, nWords, acc, fp, fp4_scratch_bytes(),
		                sCompute);
	}
	else rc = comb_muladd(a.dIn, pitch, numInputs, dIdx, dRec, recPitchAlloc, R, nWords, acc, shape, sCompute);
	if(rc) return -1;
	processingAdd = true;
	a.hasCustom = false;
	finish_area(areaIdx, numInputs);
	return 0;
}

void Engine::finish_area(unsigned areaIdx, unsigned numInputs) {
	notify_after(sCompute, [this, areaIdx, numInputs] {
		Area& a = staging[areaIdx];
		stagingActiveCount--;
		{
			std::lock_guard<std::mutex> lk(a.m);
			a.active = false;
		}
		a.cv.notify_all();
		if(progressFn) progressFn(progressUser, numInputs);
	});
}

int Engine::do_end(const Req& r) {
	const unsigned R = (unsigned)outputExponents.size();
	if(processingAdd && R) {
		uint8_t* sp = reinterpret_cast<uint8_t*>(dScratch);
		sp += round_up(std::max(idx_bytes(R, batchPad), tc_scratch_bytes(R, batchPad)), 256);
		sp += round_up((size_t)R * batchPad * 2, 256);
		unsigned long long* dCk = reinterpret_cast<unsigned long long*>(sp);
		sp += round_up(std::max<size_t>(R, batchPad) * 8, 256);
		uint8_t* dFlags = sp;
		if(rows_cksum(dRec, recPitchAlloc, R, nullptr, currentSliceSize, dCk, 1, dFlags, gt, sCompute)) return -1;
		P2C_CUDA_TRY(cudaMemcpyAsync(hFlags, dFlags, R, cudaMemcpyDeviceToHost, sCompute));
	}
	par2cuda_done_fn cb = r.cb;
	void* user = r.user;
	notify_after(sCompute, [cb, user] { if(cb) cb(user, 0); });
	return 0;
}

int Engine::do_output(const Req& r) {
	const size_t S = currentSliceSize;
	if(!processingAdd) {
		memset(const_cast<void*>(r.buf), 0, S); // nothing computed -> zeros (controller.cpp:376-382)
		if(r.cb) r.cb(r.user, 1);
		return 0;
	}
	// ordered after the end-of-input verification on the compute stream
	cudaEvent_t ev = take_event();
	P2C_CUDA_TRY(cudaEventRecord(ev, sCompute));
	P2C_CUDA_TRY(cudaStreamWaitEvent(sOut, ev, 0));
	give_event(ev);
	const uint16_t* src = dRec + (size_t)r.slot * recPitchAlloc;
	void* out = const_cast<void*>(r.buf);
	const unsigned slot = r.slot;
	par2cuda_done_fn cb = r.cb;
	void* user = r.user;
	if(is_pinned(out)) {
		// asynchronous: the verdict callback fires from the notifier thread once
		// the copy (and the verification it is ordered after) has completed
		P2C_CUDA_TRY(cudaMemcpyAsync(out, src, S, cudaMemcpyDefault, sOut));
		notify_after(sOut, [this, slot, cb, user] { if(cb) cb(user, hFlags ? hFlags[slot] : 0); });
		return 0;
	}
	if(hOutBounceBytes < S) {
		P2C_CUDA_TRY(cudaStreamSynchronize(sOut));
		if(hOutBounce) cudaFreeHost(hOutBounce);
		hOutBounce = nullptr;
		P2C_CUDA_TRY(cudaHostAlloc(&hOutBounce, S, cudaHostAllocDefault));
		hOutBounceBytes = S;
	}
	P2C_CUDA_TRY(cudaMemcpyAsync(hOutBounce, src, S, cudaMemcpyDeviceToHost, sOut));
	P2C_CUDA_TRY(cudaStreamSynchronize(sOut));
	memcpy(out, hOutBounce, S);
	if(cb) cb(user, hFlags ? hFlags[slot] : 0);
	return 0;
}

int Engine::info(par2cuda_info* o) {
	memset(o, 0, sizeof(*o));
	o->device = device;
	cudaDeviceProp p;
	if(cudaGetDeviceProperties(&p, device) == cudaSuccess) snprintf(o->device_name, sizeof(o->device_name), "%.127s", p.name);
	const char* names[] = {"auto", "Comb (XOR-combination tables)", "Xor (LOP3 bit masks)", "Nibble tables",
	                       "Tensor (tcgen05 GF(2) bit-matrix, e4m3)", "Tensor (tcgen05 GF(2) bit-matrix, block-scaled e2m1)"};
	snprintf(o->method_desc, sizeof(o->method_desc), "%s", names[method >= 0 && method <= 5 ? method : 0]);
	o->staging_count = (unsigned)staging.size();
	o->staging_size = inputBatchSize;
	o->min_staging_size = minInBatchSize;
	o->chunk_size = P2C_TILE_WORDS * 2;
	o->slice_mem = row_pitch(allocSliceSize) * 2;
	o->slice_size = currentSliceSize;
	o->num_output_slices = (unsigned)outputExponents.size();
	o->batches_started = statBatchesStarted;
	o->device_bytes = (size_t)staging.size() * batchPad * stagingPitch * 2 + recRowsAlloc * recPitchAlloc * 2 + scratchBytes;
	return 0;
}

} // namespace p2c
