"""Failure detection without faulting the GPU.

  * A bounded device wait runs out: par2cuda_wait_selftest makes one warp
    wait, with the kernels' own wait helper, on an mbarrier that nothing
    arrives on.  The wait gives up after its poll limit, the kernel returns,
    par2cuda_device_error() reports 1 (then 0 once read), and the context
    stays usable for a normal bit-exact recovery afterwards.
  * Allocation failure: requests the device cannot hold (a multi-TiB
    staging area or recovery buffer; the allocation fails at once and holds
    nothing) surface as the reference's "Failed to allocate memory"
    (src/gf.cc:351-354, 489-490), and the backend stays usable.
  * Corruption: covered by test_gpu_parity.py's flipped-bit verdict test.
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from parpar_gb300 import _lib, synth
from parpar_gb300.gfproc import GfProc, GfProcError, create_recovery

pytestmark = pytest.mark.gpu


def small_recovery_ok():
    """A recovery through the backend (its own threads) and a launch from this
    thread both still work: a failed allocation must not leave a stale error
    behind for the next launch check on the calling thread."""
    import torch
    L = _lib.load()
    d = torch.empty(4096, dtype=torch.uint8, device="cuda")
    if L.par2cuda_synth_fill(d.data_ptr(), 4096, 1, 4096, 1, 0, None) != 0:
        return False
    torch.cuda.synchronize()
    if not np.array_equal(d.cpu().numpy(), synth.slices(1, 0, 1, 4096)[0]):
        return False
    x = synth.slices(3, 0, 12, 3000)
    out, valid = create_recovery(x, np.full(12, 3000), np.arange(12), [0, 1, 5])
    return valid.all() and np.array_equal(out, O.recover(x, np.full(12, 3000), np.arange(12), [0, 1, 5]))


@pytest.mark.parametrize("polls", [1, 1000, 1 << 16])
def test_bounded_wait_gives_up_and_reports(polls):
    L = _lib.load()
    assert L.par2cuda_device_error() in (0, 1)     # clear anything earlier
    gave_up = ctypes.c_int(-1)
    secs = ctypes.c_double(-1)
    assert L.par2cuda_wait_selftest(polls, ctypes.byref(gave_up), ctypes.byref(secs)) == 0
    assert gave_up.value == 1
    assert 0 <= secs.value < 5.0
    assert L.par2cuda_device_error() == 1
    assert L.par2cuda_device_error() == 0          # read clears it
    assert small_recovery_ok()                     # the context is still usable
    assert L.par2cuda_device_error() == 0


def test_wait_selftest_rejects_bad_limits():
    L = _lib.load()
    g, s = ctypes.c_int(), ctypes.c_double()
    assert L.par2cuda_wait_selftest(0, ctypes.byref(g), ctypes.byref(s)) < 0
    assert L.par2cuda_wait_selftest((1 << 22) + 1, ctypes.byref(g), ctypes.byref(s)) < 0


def test_staging_allocation_failure_is_failed_to_allocate():
    # 2^40-byte slices: eight staging rows per area cannot be allocated
    with pytest.raises(GfProcError, match="Failed to allocate memory"):
        GfProc(1 << 40)
    assert small_recovery_ok()


def test_recovery_allocation_failure_is_failed_to_allocate():
    g = GfProc(1 << 20, input_batchsize=8)
    try:
        # 65534 recovery rows of 1 MiB fit (64 GiB) on this device class;
        # 2^30-byte rows via setCurrentSliceSize do not
        g.set_recovery_slices(list(range(4)))
        with pytest.raises(GfProcError, match="Failed to allocate memory"):
            g.set_current_slice_size(1 << 42)
    finally:
        g.close()
    assert small_recovery_ok()
