// PAR2ProcCUDA backend object (see engine.cu).
#pragma once
#include "common.cuh"
#include "kernels.h"
#include "../../include/par2cuda.h"

#include <atomic>
#include <condition_variable>
#include <deque>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace p2c {

struct Area {
	uint16_t* dIn = nullptr;     // batchPad rows x stagingPitch words
	uint8_t* hBounce = nullptr;  // pinned bounce rows for pageable sources
	size_t bounceBytes = 0;
	uint8_t* hDesc = nullptr;    // pinned batch descriptor (lens, logs, coefficients, exponents)
	uint8_t* dDesc = nullptr;
	size_t descBytes = 0;
	std::vector<uint16_t> logs;   // per slot: PAR2 input log, 0 = explicit coefficients
	std::vector<uint32_t> lens;   // per slot: bytes supplied
	std::vector<uint16_t> custom; // [slot][R] explicit coefficients
	bool hasCustom = false;
	std::atomic<bool> active{false};
	std::mutex m;
	std::condition_variable cv;
};

struct Req {
	enum Kind { ADD, DUMMY, FILL, FLUSH, END, OUTPUT, STOP } kind;
	const void* buf = nullptr;
	size_t size = 0;
	unsigned area = 0, slot = 0, submit = 0;
	par2cuda_done_fn cb = nullptr;
	void* user = nullptr;
};

struct Note {
	cudaEvent_t ev = nullptr;
	std::function<void()> fn;
	bool stop = false;
};

class Engine {
public:
	Engine(int device, unsigned areas);
	~Engine();
	int start();
	void shutdown();

	int init(int method, unsigned inputBatch);
	int set_slice_size(size_t s);
	int set_current_slice_size(size_t s);
	int set_recovery_slices(unsigned n, const uint16_t* exps);
	void set_min_input_batch(unsigned n) { minInBatchSize = n ? n : inputBatchSize; }
	void set_progress(par2cuda_progress_fn fn, void* user) { progressFn = fn; progressUser = user; }
	void set_shape(int s) { shape = s; }

	int can_add() const;
	int wait_for_add();
	int add_input(const void* buf, size_t size, int inputNum, const uint16_t* coeffs, bool flush,
	              par2cuda_done_fn cb, void* user, bool dummy = false);
	int fill_input(const void* buf);
	int flush();
	int end_input(par2cuda_done_fn cb, void* user);
	int get_output(unsigned index, void* out, par2cuda_done_fn cb, void* user);
	// checksum verdict of output `index` once end_input has completed (after sync)
	int output_valid(unsigned index);
	void discard_output() { processingAdd = false; }
	bool has_added() const { return processingAdd; }
	bool is_empty() const { return stagingActiveCount.load() == 0; }
	int sync();
	int free_processing_mem();
	int info(par2cuda_info* o);

private:
	int device;
	GfTables gt{};
	int method = 1, shape = 0;
	size_t sliceSize = 0, allocSliceSize = 0, currentSliceSize = 0;
	unsigned inputBatchSize = 0, batchPad = 0, minInBatchSize = 0;
	unsigned currentStagingArea = 0, currentStagingInputs = 0, statBatchesStarted = 0;
	std::atomic<unsigned> stagingActiveCount{0};
	bool processingAdd = false, initialised = false, running = false;
	std::vector<uint16_t> outputExponents;
	std::vector<Area> staging;
	size_t stagingPitch = 0;

	uint16_t* dRec = nullptr;
	size_t recRowsAlloc = 0, recPitchAlloc = 0;
	void* dScratch = nullptr;
	size_t scratchBytes = 0;
	uint8_t* hFlags = nullptr;
	uint8_t* hOutBounce = nullptr;
	size_t hOutBounceBytes = 0;

	cudaStream_t sCopy = nullptr, sCompute = nullptr, sOut = nullptr;
	par2cuda_progress_fn progressFn = nullptr;
	void* progressUser = nullptr;
	std::atomic<int> lastAsyncError{0};

	std::thread transferThread, notifyThread;
	std::mutex qm, nm, em;
	std::condition_variable qcv, ncv, idleCv, nIdleCv;
	std::deque<Req> tq;
	std::deque<Note> nq;
	bool transferBusy = false, notifyBusy = false;
	std::vector<cudaEvent_t> eventPool;

	size_t desc_bytes() const;
	int alloc_staging();
	int alloc_desc();
	int alloc_processing();
	size_t fp4_scratch_bytes() const;
	void free_staging();
	void free_processing();
	void wait_idle();
	static uint16_t host_exp(uint32_t e);

	void enqueue(const Req& r);
	void notify_after(cudaStream_t st, std::function<void()> fn);
	cudaEvent_t take_event();
	void give_event(cudaEvent_t e);
	void transfer_loop();
	void notify_loop();
	int do_copy(const Req& r);
	int run_kernel(unsigned area, unsigned numInputs);
	void finish_area(unsigned area, unsigned numInputs);
	int do_end(const Req& r);
	int do_output(const Req& r);
};

} // namespace p2c
