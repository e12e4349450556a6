"""The reference's own CPU core as a checker — test infrastructure, not product code.

ParPar's gf16/ + hasher/ sources are read from the reference tree named by the
environment variable PARPAR_REFERENCE (the checkout of Ravencentric/ParPar;
default: the read-only checkout at DEFAULT_REFERENCE, when present) and
staged, unmodified, into oracle/_ref/src/.  That folder is git-ignored: the
sources never enter the repository's history, but they travel with the working
tree to the GPU host, which is an aarch64 machine where the x86 objects built
here cannot run.  oracle/ref.mk then compiles the staged tree on whatever host
it is on (here, and on the GPU host from build()), with binding.gyp's per-file
ISA flags, into:

  oracle/_ref/libparref.so       the reference core + oracle/ref_shim.cpp: pins
                                 the oracle, generates tests/golden/, and is the
                                 timed CPU path of `bench.py --impl reference`
                                 (no library of this repository is linked in);
  oracle/_ref/libparref_cuda.so  the same core + the PAR2ProcCUDA adapter
                                 (parpar_gb300/adapter/) + oracle/adapter_shim.cpp,
                                 linked with libpar2cuda.so: drives the CUDA
                                 backend through the reference's own PAR2Proc.

Only tests/, __graft_entry__ (building and smoke) and bench.py's CPU legs use it.
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
REF_OUT = os.path.join(HERE, "_ref")
STAGED = os.path.join(REF_OUT, "src")
REF_LIB = os.path.join(REF_OUT, "libparref.so")
REF_CUDA_LIB = os.path.join(REF_OUT, "libparref_cuda.so")

# what the CPU controller, the coefficient tables, the checksum and the hashers
# need (binding.gyp targets parpar_gf minus the OpenCL files, gf16*, hasher*)
_SKIP = ("controller_ocl.h", "controller_ocl.cpp", "controller_ocl_init.cpp", "xor_jit_stub_masm64.asm")
_SRC_HEADERS = ("platform.h", "cpuid.h", "hedley.h", "stdint.h")


DEFAULT_REFERENCE = "/root/reference"


def reference_dir() -> str | None:
    """The reference checkout named by PARPAR_REFERENCE (else the read-only
    checkout at DEFAULT_REFERENCE), if it holds gf16/."""
    for d in (os.environ.get("PARPAR_REFERENCE"), DEFAULT_REFERENCE):
        if d and os.path.isfile(os.path.join(d, "gf16", "controller.h")):
            return d
    return None


def stage(ref: str | None = None) -> bool:
    """Copies the needed reference sources into oracle/_ref/src/ (git-ignored).
    Returns False when no reference tree is available."""
    ref = ref or reference_dir()
    if not ref:
        return False
    for sub in ("gf16", "hasher"):
        os.makedirs(os.path.join(STAGED, sub), exist_ok=True)
        for f in sorted(os.listdir(os.path.join(ref, sub))):
            p = os.path.join(ref, sub, f)
            if f in _SKIP or not os.path.isfile(p) or not f.endswith((".c", ".cpp", ".h")):
                continue
            _copy_if_changed(p, os.path.join(STAGED, sub, f))
    os.makedirs(os.path.join(STAGED, "src"), exist_ok=True)
    for f in _SRC_HEADERS:
        _copy_if_changed(os.path.join(ref, "src", f), os.path.join(STAGED, "src", f))
    return True


def _copy_if_changed(src: str, dst: str) -> None:
    if os.path.exists(dst) and os.path.getsize(dst) == os.path.getsize(src):
        with open(src, "rb") as a, open(dst, "rb") as b:
            if a.read() == b.read():
                return
    shutil.copyfile(src, dst)


def staged() -> bool:
    return os.path.isfile(os.path.join(STAGED, "gf16", "controller.h"))


def build(with_cuda: bool = True) -> dict:
    """Compiles the staged reference core (and, when libpar2cuda.so exists,
    the adapter library).  Returns {"ref": path|None, "ref_cuda": path|None,
    "error": message|None}; never raises for a compile failure, so that a host
    where the reference does not build still gets the rest of the checker."""
    out = {"ref": None, "ref_cuda": None, "error": None}
    if not staged():
        out["error"] = "reference sources not staged (set PARPAR_REFERENCE where the reference tree exists)"
        return out
    jobs = "-j%d" % (os.cpu_count() or 4)
    targets = ["ref"]
    cuda_lib = os.path.join(ROOT, "parpar_gb300", "libpar2cuda.so")
    if with_cuda and os.path.exists(cuda_lib):
        targets.append("ref_cuda")
    for t in targets:
        r = subprocess.run(["make", "-s", "-f", os.path.join("oracle", "ref.mk"), "REF=" + os.path.relpath(STAGED, ROOT),
                            jobs, t], cwd=ROOT, capture_output=True, text=True)
        if r.returncode != 0:
            out["error"] = "%s build failed: %s" % (t, (r.stderr or r.stdout).strip()[-2000:])
            break
        out[t] = REF_LIB if t == "ref" else REF_CUDA_LIB
    return out
