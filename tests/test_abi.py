"""The C-ABI library loads and exports every function include/*.h declares;
SeqPair keeps the reference's 56-byte layout.  No compute calls (CPU only)."""
import ctypes
import glob
import os
import re

import numpy as np

import tal_bsw
from tal_bsw.seqpair import SEQPAIR_DTYPE, SEQPAIR_FIELDS

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b(tal_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_headers_declare_entry_points():
    names = _declared()
    for must in ("tal_bsw_create", "tal_bsw_destroy", "tal_bsw_scores", "tal_bsw_scores_device",
                 "tal_bsw_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(tal_bsw.CORE_LIB)
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_seqpair_layout():
    assert SEQPAIR_DTYPE.itemsize == 56
    assert list(SEQPAIR_DTYPE.names) == list(SEQPAIR_FIELDS)
    assert [SEQPAIR_DTYPE.fields[f][1] for f in SEQPAIR_FIELDS] == list(range(0, 56, 4))


def test_create_without_gpu_fails_cleanly():
    """On a machine without a GB300 the constructor raises (no CPU fallback)."""
    import torch
    if torch.cuda.is_available():
        return
    try:
        tal_bsw.BandedPairWiseSW(6, 1, 6, 1, 100, 5, None, 1, 4, 1)
    except tal_bsw.TalBswError as e:
        assert e.status == tal_bsw.api.TAL_ENODEV
    else:
        raise AssertionError("expected TAL_ENODEV")


def test_bad_params_rejected_before_device():
    lib = tal_bsw.api.core_lib()
    p = tal_bsw.api._Params(6, 0, 6, 1, 100, 5, 1, 4)   # e_del = 0
    h = ctypes.c_void_p()
    assert lib.tal_bsw_create(ctypes.byref(p), 0, ctypes.byref(h)) == tal_bsw.api.TAL_EINVAL


def test_ctypes_structs_match_the_header(tmp_path):
    """The Python mirrors of the serving structs have the C layout (sizes and
    field offsets as gcc lays out include/tal_bsw.h)."""
    import subprocess
    from tal_bsw.api import RequestInfo, ServerConfig, ServerStats, _Params
    from tal_bsw.sw import _SwParams
    import numpy as np
    from tal_bsw.swdata import SW_DTYPE

    class _SwPair(ctypes.Structure):
        _fields_ = [(n, {"<i4": ctypes.c_int32, "<i2": ctypes.c_int16}[SW_DTYPE.fields[n][0].str])
                    for n in SW_DTYPE.names]
        _pack_ = 1
    from tal_bsw.chain import _ChainParams
    from tal_bsw.chaindata import ANCHOR_DTYPE

    class _Anchor(ctypes.Structure):
        _fields_ = [("r", ctypes.c_uint64), ("q", ctypes.c_int32), ("l", ctypes.c_int32)]
    assert ctypes.sizeof(_Anchor) == ANCHOR_DTYPE.itemsize
    assert [ANCHOR_DTYPE.fields[n][1] for n in ANCHOR_DTYPE.names] == \
        [getattr(_Anchor, n).offset for n, _ in _Anchor._fields_]
    from tal_bsw.extend import _ExtParams
    from tal_bsw.seeddata import REGION_DTYPE, SEED_DTYPE

    def _mirror(dt):
        m = {"<i4": ctypes.c_int32, "<i8": ctypes.c_int64}

        class _S(ctypes.Structure):
            _fields_ = [(n, m[dt.fields[n][0].str]) for n in dt.names]
        assert ctypes.sizeof(_S) == dt.itemsize
        assert [dt.fields[n][1] for n in dt.names] == [getattr(_S, n).offset for n in dt.names]
        return _S
    structs = {"tal_bsw_server_config": ServerConfig, "tal_bsw_request_info": RequestInfo,
               "tal_bsw_server_stats": ServerStats, "tal_bsw_params": _Params,
               "tal_sw_params": _SwParams, "tal_sw_pair": _SwPair,
               "tal_chain_params": _ChainParams, "tal_anchor": _Anchor,
               "tal_extend_params": _ExtParams, "tal_seed": _mirror(SEED_DTYPE),
               "tal_region": _mirror(REGION_DTYPE)}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "tal_bsw.h"', '#include "tal_sw.h"',
             '#include "tal_chain.h"', '#include "tal_extend.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), "-o", str(exe), str(src)])
    got = {}
    for line in subprocess.check_output([str(exe)]).decode().splitlines():
        c, f, v = line.split()
        got[(c, f)] = int(v)
    for cname, py in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for f, _ in py._fields_:
            assert got[(cname, f)] == getattr(py, f).offset, (cname, f)


def test_precision_constants_match_the_header():
    """The Python constants for the precision argument equal the header's
    enum (TAL_BSW_AUTO / _8 / _16 and the TAL_BSW_GROUPED flag)."""
    src = open(os.path.join(ROOT, "include", "tal_bsw.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    vals = {m.group(1): int(m.group(2), 0) for m in re.finditer(r"\b(TAL_BSW_\w+)\s*=\s*(0x[0-9a-fA-F]+|\d+)", src)}
    assert vals["TAL_BSW_AUTO"] == tal_bsw.api.AUTO
    assert vals["TAL_BSW_8"] == tal_bsw.api.BITS8
    assert vals["TAL_BSW_16"] == tal_bsw.api.BITS16
    assert vals["TAL_BSW_GROUPED"] == tal_bsw.api.GROUPED
    assert vals["TAL_BSW_GROUPED"] & 0xff == 0


def test_cpp_dropin_header_compiles_and_links():
    """The C++ drop-in header (include/bandedSWA_gb300.h) compiles with g++
    -Wall -Werror (its SeqPair layout static_asserts included) and a caller of
    the reference's interface links against libtal_bsw.so.  Running it needs a
    GB300 (tests/test_gpu_cpp_dropin.py)."""
    import tempfile
    import cpp_dropin
    with tempfile.TemporaryDirectory() as d:
        exe = cpp_dropin.build(d)
        assert os.path.exists(exe)
