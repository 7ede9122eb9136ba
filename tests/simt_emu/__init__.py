"""ctypes driver for the SIMT emulator (emu.cpp): runs the CUDA kernel source
compiled for the host, one thread per lane.  Test infrastructure only."""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
CSRC = os.path.join(ROOT, "trans-omics-acceleration-library_gb300", "csrc")
SO = os.path.join(ROOT, "tests", "simt_emu", "_build", "libbsw_emu.so")
_lib = None


def build(force=False):
    srcs = [os.path.join(HERE, "emu.cpp"), os.path.join(HERE, "fake", "cuda_runtime.h"),
            os.path.join(CSRC, "bsw_kernel.cuh"), os.path.join(CSRC, "bsw_lane.cuh")]
    if force or not os.path.exists(SO) or os.path.getmtime(SO) < max(os.path.getmtime(s) for s in srcs):
        os.makedirs(os.path.dirname(SO), exist_ok=True)
        subprocess.check_call(["g++", "-std=c++20", "-O1", "-fPIC", "-shared", "-pthread", "-w",
                               "-I" + os.path.join(HERE, "fake"), "-I" + CSRC, "-o", SO,
                               os.path.join(HERE, "emu.cpp")])
    return SO


def run(pairs, ref, qer, w, params, bits=16, K=4, warps=1, wpair=None, G=32):
    """Scores a copy of pairs with the emulated kernel; returns (pairs, err_flags, err_index)."""
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        _lib.emu_bsw_run.restype = ctypes.c_int
    out = np.ascontiguousarray(pairs).copy()
    kp = np.array([params[k] for k in ("o_del", "e_del", "o_ins", "e_ins", "zdrop", "end_bonus", "a", "b")],
                  np.int32)
    ef = ctypes.c_int(0)
    ei = ctypes.c_longlong(0)
    ref = np.ascontiguousarray(ref)
    qer = np.ascontiguousarray(qer)
    wp = None if wpair is None else np.ascontiguousarray(wpair, np.int32)
    vp = ctypes.c_void_p
    _lib.emu_bsw_run(vp(out.ctypes.data), vp(ref.ctypes.data), ctypes.c_longlong(0),
                     ctypes.c_longlong(ref.shape[0]), vp(qer.ctypes.data), ctypes.c_longlong(0),
                     ctypes.c_longlong(qer.shape[0]), int(out.shape[0]), int(w),
                     None if wp is None else vp(wp.ctypes.data), int(bits), vp(kp.ctypes.data),
                     int(G), int(K), int(warps), ctypes.byref(ef), ctypes.byref(ei))
    return out, ef.value, ei.value
