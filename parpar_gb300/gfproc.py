"""Host-side mirror of ParPar's GfProc (src/gf.cc:236-733) over the CUDA backend.

Same method names, argument meaning and error behaviour as the addon's
JavaScript-facing class, so code written against GfProc (lib/par2.js
GFWrapper, examples/simple.js) reads the same:

    g = GfProc(slice_size)                 # GfProc::New, src/gf.cc:253-385
    g.set_recovery_slices([0, 1, 2])       # SetRecoverySlices :461-492
    g.add(idx, buffer, cb) -> bool         # AddSlice :570-622 (False = backend full)
    g.end(cb)                              # EndInput :624-648
    g.get(idx, out, cb(idx, valid, out))   # GetOutputSlice :650-695
    g.set_current_slice_size(n)            # SetCurrentSliceSize :439-460
    g.info(); g.free_mem(); g.close()

Errors raise GfProcError with the addon's messages ("Slice size is invalid",
"Input index not valid", ...).  Callbacks run on the backend's notifier
thread.  Everything runs through libpar2cuda.so; there is no CPU path.
"""
from __future__ import annotations

import ctypes
import threading

import numpy as np

from . import _lib


class GfProcError(ValueError):
    pass


def _buf_ptr(buf):
    """(pointer, nbytes, keepalive) for numpy arrays, bytes-like objects and torch tensors."""
    if hasattr(buf, "data_ptr") and hasattr(buf, "element_size"):  # torch tensor (host)
        return buf.data_ptr(), buf.numel() * buf.element_size(), buf
    a = np.frombuffer(buf, dtype=np.uint8) if not isinstance(buf, np.ndarray) else buf
    if not a.flags["C_CONTIGUOUS"]:
        raise GfProcError("buffer must be contiguous")
    return a.ctypes.data, a.nbytes, a


class GfProc:
    def __init__(self, slice_size: int, method: str | int = "auto", input_batchsize: int = 0,
                 staging_areas: int = 2, device: int = 0, input_minbatchsize: int = 0):
        if slice_size < 2 or slice_size & 1:
            raise GfProcError("Slice size is invalid")
        if input_batchsize > 32768:
            raise GfProcError("Input batchsize is invalid")
        if staging_areas < 1 or staging_areas > 32768:
            raise GfProcError("Staging area count is invalid")
        if input_batchsize * staging_areas > 65536:
            raise GfProcError("Staging area too large")
        self._L = _lib.load()
        self._ctx = ctypes.c_void_p()
        _lib.check(self._L.par2cuda_create(device, staging_areas, ctypes.byref(self._ctx)), "create")
        m = _lib.METHOD_NAMES[method] if isinstance(method, str) else int(method)
        _lib.check(self._L.par2cuda_set_slice_size(self._ctx, slice_size), "setSliceSize")
        if self._L.par2cuda_init(self._ctx, m, input_batchsize) < 0:
            self._L.par2cuda_destroy(self._ctx)
            raise GfProcError("Failed to allocate memory")
        if input_minbatchsize:
            self._L.par2cuda_set_min_input_batch(self._ctx, input_minbatchsize)
        self.slice_size = slice_size
        self.current_slice_size = slice_size
        self.num_recovery = 0
        self.is_running = False
        self.is_closed = False
        self.has_output = False
        self._pending_discard = True
        self._keep = {}
        self._keep_lock = threading.Lock()
        self._next_token = 1
        self._progress = None
        self._progress_cfn = None
        # one C callback trampoline for every completion
        self._done_cfn = _lib.DONE_FN(self._on_done)

    # ------------------------------------------------------------ plumbing
    def _register(self, fn):
        with self._keep_lock:
            tok = self._next_token
            self._next_token += 1
            self._keep[tok] = fn
        return tok

    def _on_done(self, user, status):
        with self._keep_lock:
            fn = self._keep.pop(user, None)
        if fn is not None:
            fn(status)

    def _check_open(self):
        if self.is_closed:
            raise GfProcError("Already closed")

    # ------------------------------------------------------------ API
    def set_current_slice_size(self, size: int):
        self._check_open()
        if self.is_running:
            raise GfProcError("Cannot change params whilst running")
        if size < 2 or size & 1:
            raise GfProcError("Slice size is invalid")
        self.has_output = False
        if self._L.par2cuda_set_current_slice_size(self._ctx, size) < 0:
            raise GfProcError("Failed to allocate memory")
        self.current_slice_size = size

    def set_recovery_slices(self, exponents):
        self._check_open()
        if self.is_running:
            raise GfProcError("Cannot change params whilst running")
        exps = list(exponents)
        if len(exps) > 65534:
            raise GfProcError("Too many recovery indicies specified")
        if len(exps) < 1:
            raise GfProcError("At least one recovery index must be supplied")
        for e in exps:
            if e < 0 or e > 65534:
                raise GfProcError("Invalid recovery index supplied")
        arr = np.array(exps, dtype=np.uint16)
        self.has_output = False
        if self._L.par2cuda_set_recovery_slices(self._ctx, len(exps), arr.ctypes.data) < 0:
            raise GfProcError("Failed to allocate memory")
        self.num_recovery = len(exps)

    def set_progress_cb(self, cb=None):
        self._check_open()
        self._progress = cb
        if cb is None:
            self._progress_cfn = _lib.PROGRESS_FN(0)
        else:
            self._progress_cfn = _lib.PROGRESS_FN(lambda user, n: cb(n))
        self._L.par2cuda_set_progress_cb(self._ctx, self._progress_cfn, None)

    def add(self, idx: int, buf, cb=None, coeffs=None) -> bool:
        """Queues input slice `idx`; returns False when the backend is full
        (the caller retries after a progress callback, lib/par2.js:133-163)."""
        self._check_open()
        if not self.num_recovery:
            raise GfProcError("setRecoverySlices not yet called")
        if coeffs is None and (idx < 0 or idx > 32767):
            raise GfProcError("Input index not valid")
        ptr, n, keep = _buf_ptr(buf)
        if n > self.current_slice_size:
            raise GfProcError("Input buffer too large")
        self.is_running = True
        self.has_output = False
        if self._pending_discard:
            self._pending_discard = False
            self._L.par2cuda_discard_output(self._ctx)
        if self._L.par2cuda_can_add(self._ctx) == _lib.ADD_FULL:
            return False
        tok = self._register(lambda st, keep=keep: cb(idx, buf) if cb else None)
        if coeffs is None:
            rc = self._L.par2cuda_add_input(self._ctx, ptr, n, idx, 0, self._done_cfn, tok)
        else:
            c = np.ascontiguousarray(coeffs, dtype=np.uint16)
            if c.size != self.num_recovery:
                raise GfProcError("coefficient count must equal the number of recovery slices")
            # the backend copies the coefficient column before returning
            rc = self._L.par2cuda_add_input_coeffs(self._ctx, ptr, n, c.ctypes.data, 0, self._done_cfn, tok)
        if rc < 0:
            self._on_done(tok, -1)
            _lib.check(rc, "addInput")
        return True

    def add_sync(self, idx: int, buf, coeffs=None):
        """Blocking add: waits for room (waitForAdd) and for the copy."""
        ev = threading.Event()
        while True:
            self._L.par2cuda_wait_for_add(self._ctx)
            if self.add(idx, buf, lambda *_: ev.set(), coeffs=coeffs):
                break
        return ev

    def end(self, cb=None):
        self._check_open()
        if not self.num_recovery:
            raise GfProcError("setRecoverySlices not yet called")
        if self._pending_discard:
            self._L.par2cuda_discard_output(self._ctx)

        def fin(status):
            self.is_running = False
            self.has_output = True
            self._pending_discard = True
            if cb:
                cb()
        tok = self._register(fin)
        _lib.check(self._L.par2cuda_end_input(self._ctx, self._done_cfn, tok), "endInput")

    def end_sync(self):
        ev = threading.Event()
        self.end(ev.set)
        ev.wait()

    def get(self, idx: int, out, cb=None):
        self._check_open()
        if self.is_running:
            raise GfProcError("Cannot get output whilst running")
        if not self.has_output:
            raise GfProcError("No finalized output to retrieve")
        ptr, n, keep = _buf_ptr(out)
        if n < self.current_slice_size:
            raise GfProcError("Output buffer too small")
        if idx < 0 or idx >= self.num_recovery:
            raise GfProcError("Recovery index is not valid")
        tok = self._register(lambda st, keep=keep: cb(idx, bool(st == 1), out) if cb else None)
        _lib.check(self._L.par2cuda_get_output(self._ctx, idx, ptr, self._done_cfn, tok), "getOutput")

    def get_sync(self, idx: int, out) -> bool:
        res = {}
        ev = threading.Event()

        def done(i, valid, o):
            res["valid"] = valid
            ev.set()
        self.get(idx, out, done)
        ev.wait()
        return res["valid"]

    def sync(self):
        _lib.check(self._L.par2cuda_sync(self._ctx), "sync")

    def info(self) -> dict:
        self._check_open()
        if not self.num_recovery:
            raise GfProcError("setRecoverySlices not yet called")
        inf = _lib.Info()
        _lib.check(self._L.par2cuda_info_get(self._ctx, ctypes.byref(inf)), "info")
        return {
            "device_name": inf.device_name.decode(), "method_desc": inf.method_desc.decode(),
            "staging_count": inf.staging_count, "staging_size": inf.staging_size,
            "chunk_size": inf.chunk_size, "slice_mem": inf.slice_mem,
            "num_output_slices": inf.num_output_slices, "batches_started": inf.batches_started,
            "device_bytes": inf.device_bytes,
        }

    def free_mem(self):
        self._check_open()
        if self.is_running:
            raise GfProcError("Cannot free memory whilst running")
        self._L.par2cuda_free_processing_mem(self._ctx)
        self.has_output = False

    def close(self):
        if self.is_running:
            raise GfProcError("Cannot close whilst running")
        if self.is_closed:
            raise GfProcError("Already closed")
        self._L.par2cuda_destroy(self._ctx)
        self.is_closed = True

    def __del__(self):
        try:
            if not self.is_closed and not self.is_running:
                self._L.par2cuda_destroy(self._ctx)
                self.is_closed = True
        except Exception:
            pass


def create_recovery(inputs: np.ndarray, lens, input_nums, exps, method="auto", input_batchsize=0,
                    staging_areas=2, slice_size=None):
    """Runs one full create pass (add every input, end, get every output) and
    returns (recovery uint8[R, S], valid bool[R])."""
    inputs = np.ascontiguousarray(inputs, dtype=np.uint8)
    n, S = inputs.shape
    S = slice_size or S
    g = GfProc(S, method=method, input_batchsize=input_batchsize, staging_areas=staging_areas)
    try:
        g.set_recovery_slices(exps)
        events = []
        for i in range(n):
            events.append(g.add_sync(int(input_nums[i]), inputs[i, : int(lens[i])]))
        g.end_sync()
        for e in events:
            e.wait()
        out = np.zeros((len(exps), S), dtype=np.uint8)
        valid = np.zeros(len(exps), dtype=bool)
        for r in range(len(exps)):
            valid[r] = g.get_sync(r, out[r])
        g.close()
    except Exception:
        raise
    return out, valid
