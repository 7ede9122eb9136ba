"""Seeded synthetic seed-extension workloads (the stand-in for the pair files
read by benchmarks/bench-bsw.cpp:117-169, which the reference does not ship).

Generation runs in the host library ``libtal_bsw_synth.so`` (csrc/synth.cpp);
this module holds the workload shapes and lays the pairs out the way the
reference's callers do: one SeqPair per pair with ``idr``/``idq`` byte offsets
into a reference buffer and a query buffer.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

from ._lib import load_synth
from .seqpair import SEQPAIR_DTYPE, new_pairs


class _Cfg(ctypes.Structure):
    _fields_ = [
        ("seed", ctypes.c_uint64),
        ("len_dist", ctypes.c_int32), ("len_lo", ctypes.c_int32), ("len_hi", ctypes.c_int32),
        ("len_median", ctypes.c_double), ("len_sigma", ctypes.c_double),
        ("n_rate", ctypes.c_double),
        ("err_lo", ctypes.c_double), ("err_hi", ctypes.c_double),
        ("sub_frac", ctypes.c_double), ("ins_frac", ctypes.c_double), ("del_frac", ctypes.c_double),
        ("indel_lo", ctypes.c_int32), ("indel_hi", ctypes.c_int32),
        ("homopolymer_del_bias", ctypes.c_double),
        ("extra_lo", ctypes.c_int32), ("extra_hi", ctypes.c_int32),
        ("h0_lo", ctypes.c_int32), ("h0_hi", ctypes.c_int32),
        ("h0_cap_8bit", ctypes.c_int32), ("match", ctypes.c_int32),
        ("w_default", ctypes.c_int32), ("n_w_choices", ctypes.c_int32),
        ("w_choices", ctypes.c_int32 * 8),
    ]


FIXED, UNIFORM, LOGNORMAL = 0, 1, 2


@dataclass
class Workload:
    """One synthetic workload shape plus the scoring it is run with."""
    name: str
    n_pairs: int
    len_dist: int
    len_lo: int
    len_hi: int
    len_median: float = 0.0
    len_sigma: float = 0.0
    n_rate: float = 0.001
    err_lo: float = 0.0
    err_hi: float = 0.0
    sub_frac: float = 1.0
    ins_frac: float = 0.0
    del_frac: float = 0.0
    indel_lo: int = 1
    indel_hi: int = 1
    homopolymer_del_bias: float = 1.0
    extra_lo: int = 0
    extra_hi: int = 0
    h0_lo: int = 0
    h0_hi: int = 0
    h0_cap_8bit: bool = False
    w: int = 100
    w_choices: List[int] = field(default_factory=list)
    # scoring (bench-bsw.cpp:40-44, :215): a, b, o_del, e_del, o_ins, e_ins
    a: int = 1
    b: int = 4
    o_del: int = 6
    e_del: int = 1
    o_ins: int = 6
    e_ins: int = 1
    zdrop: int = 100
    end_bonus: int = 5
    bits: int = 16          # 16, 8, or 0 = route each pair by the 8-bit envelope
    seed: int = 0

    def params(self) -> Dict[str, int]:
        return dict(o_del=self.o_del, e_del=self.e_del, o_ins=self.o_ins, e_ins=self.e_ins,
                    zdrop=self.zdrop, end_bonus=self.end_bonus, a=self.a, b=self.b)

    def scaled(self, n_pairs: int, seed: Optional[int] = None) -> "Workload":
        d = dict(self.__dict__)
        d["n_pairs"] = int(n_pairs)
        d["w_choices"] = list(self.w_choices)
        if seed is not None:
            d["seed"] = int(seed)
        return Workload(**d)

    def _cfg(self) -> _Cfg:
        c = _Cfg()
        c.seed = self.seed
        c.len_dist, c.len_lo, c.len_hi = self.len_dist, self.len_lo, self.len_hi
        c.len_median, c.len_sigma = self.len_median, self.len_sigma
        c.n_rate = self.n_rate
        c.err_lo, c.err_hi = self.err_lo, self.err_hi
        c.sub_frac, c.ins_frac, c.del_frac = self.sub_frac, self.ins_frac, self.del_frac
        c.indel_lo, c.indel_hi = self.indel_lo, self.indel_hi
        c.homopolymer_del_bias = self.homopolymer_del_bias
        c.extra_lo, c.extra_hi = self.extra_lo, self.extra_hi
        c.h0_lo, c.h0_hi = self.h0_lo, self.h0_hi
        c.h0_cap_8bit = 1 if self.h0_cap_8bit else 0
        c.match = self.a
        c.w_default = self.w
        c.n_w_choices = len(self.w_choices)
        for i, v in enumerate(self.w_choices[:8]):
            c.w_choices[i] = v
        return c


def _indel_split(sub: float, indel: float):
    tot = sub + indel
    return tot, sub / tot, indel / tot / 2, indel / tot / 2


def _c1(**kw) -> Workload:
    tot, s, i, d = _indel_split(0.02, 0.002)
    base = dict(name="c1_151bp", n_pairs=100_000, len_dist=FIXED, len_lo=151, len_hi=151,
                n_rate=0.001, err_lo=tot, err_hi=tot, sub_frac=s, ins_frac=i, del_frac=d,
                indel_lo=1, indel_hi=3, extra_lo=0, extra_hi=20, h0_lo=19, h0_hi=60,
                w=100, zdrop=100, bits=0, seed=101)
    base.update(kw)
    return Workload(**base)


WORKLOADS: Dict[str, Workload] = {}


def _register(w: Workload) -> Workload:
    WORKLOADS[w.name] = w
    return w


# 100,000 pairs, query 151 bp.  151 >= 128 puts every pair outside the 8-bit
# envelope, so the routing rule sends all of them to the 16-bit kernel.
C1 = _register(_c1())
# The same generator with the query at U[20,107] so len1 <= 127 and h0 capped
# at 127 - min(len1, len2): every pair is 8-bit eligible (getScores8).
C1_8 = _register(_c1(name="c1_8bit", len_dist=UNIFORM, len_lo=20, len_hi=107,
                     h0_cap_8bit=True, bits=8, seed=102))
_t2 = _indel_split(0.04, 0.005)
# 1,000,000 pairs, query U[100,300], 4% substitutions + 0.5% 1-5 bp indels,
# len1 = len2 + U[0,40], h0 ~ U[30,250]; getScores16.
C2 = _register(Workload(name="c2_16bit", n_pairs=1_000_000, len_dist=UNIFORM, len_lo=100,
                        len_hi=300, n_rate=0.001, err_lo=_t2[0], err_hi=_t2[0],
                        sub_frac=_t2[1], ins_frac=_t2[2], del_frac=_t2[3], indel_lo=1,
                        indel_hi=5, extra_lo=0, extra_hi=40, h0_lo=30, h0_hi=250, w=100,
                        zdrop=100, bits=16, seed=202))
# 10,000,000 pairs, lognormal query (median 120, sigma 0.8) clipped to
# [20, 2000], per-pair error U[1%, 8%] (80% substitutions, 20% 1-5 bp indels),
# len1 = len2 + U[0,40], band w per pair from {20, 50, 100}, h0 ~ U[19,250];
# each pair routed to 8 or 16 bit.
C3 = _register(Workload(name="c3_mixed", n_pairs=10_000_000, len_dist=LOGNORMAL, len_lo=20,
                        len_hi=2000, len_median=120.0, len_sigma=0.8, n_rate=0.001,
                        err_lo=0.01, err_hi=0.08, sub_frac=0.8, ins_frac=0.1, del_frac=0.1,
                        indel_lo=1, indel_hi=5, extra_lo=0, extra_hi=40, h0_lo=19, h0_hi=250,
                        w=100, w_choices=[20, 50, 100], zdrop=100, bits=0, seed=303))
# 200,000 long-read pairs, query U[1000,5000], 10% errors (5% substitutions,
# 2.5% 1 bp insertions, 2.5% 1 bp deletions, deletions 3x likelier inside
# homopolymer runs), len1 = len2 + U[0,500], w = 500, zdrop = 400, h0 ~ U[50,500].
C4 = _register(Workload(name="c4_long", n_pairs=200_000, len_dist=UNIFORM, len_lo=1000,
                        len_hi=5000, n_rate=0.001, err_lo=0.10, err_hi=0.10, sub_frac=0.5,
                        ins_frac=0.25, del_frac=0.25, indel_lo=1, indel_hi=1,
                        homopolymer_del_bias=3.0, extra_lo=0, extra_hi=500, h0_lo=50,
                        h0_hi=500, w=500, zdrop=400, bits=16, seed=404))


@dataclass
class Batch:
    """A generated slice of a workload, laid out like the reference's inputs."""
    pairs: np.ndarray        # SEQPAIR_DTYPE records (idr/idq/len1/len2/h0 set)
    ref: np.ndarray          # uint8 reference bases
    qer: np.ndarray          # uint8 query bases
    w: np.ndarray            # int32 band per pair
    workload: Workload

    @property
    def n(self) -> int:
        return int(self.pairs.shape[0])


def generate(wl: Workload, n: Optional[int] = None, first: int = 0, nthreads: int = 0,
             slack: int = 64) -> Batch:
    """Generate pairs [first, first + n) of workload ``wl``.

    The sequence buffers get ``slack`` spare bytes at the end (the reference's
    callers over-allocate too); offsets are int32, as in SeqPair, so one batch
    holds at most 2 GiB of bases per buffer.
    """
    lib = load_synth()
    n = wl.n_pairs if n is None else int(n)
    cfg = wl._cfg()
    len1 = np.zeros(n, np.int32)
    len2 = np.zeros(n, np.int32)
    h0 = np.zeros(n, np.int32)
    w = np.zeros(n, np.int32)
    p32 = ctypes.POINTER(ctypes.c_int32)
    rc = lib.tal_synth_plan(ctypes.byref(cfg), ctypes.c_int64(first), ctypes.c_int64(n),
                            len1.ctypes.data_as(p32), len2.ctypes.data_as(p32),
                            h0.ctypes.data_as(p32), w.ctypes.data_as(p32), nthreads)
    if rc != 0:
        raise RuntimeError("tal_synth_plan failed")
    ref_off = np.zeros(n, np.int64)
    qer_off = np.zeros(n, np.int64)
    if n:
        ref_off[1:] = np.cumsum(len1[:-1], dtype=np.int64)
        qer_off[1:] = np.cumsum(len2[:-1], dtype=np.int64)
    rtot = int(ref_off[-1] + len1[-1]) if n else 0
    qtot = int(qer_off[-1] + len2[-1]) if n else 0
    if rtot >= 2**31 or qtot >= 2**31:
        raise ValueError("batch exceeds the int32 idr/idq range; generate it in slices")
    ref = np.zeros(rtot + slack, np.uint8)
    qer = np.zeros(qtot + slack, np.uint8)
    p64 = ctypes.POINTER(ctypes.c_int64)
    pu8 = ctypes.POINTER(ctypes.c_uint8)
    if n:
        rc = lib.tal_synth_fill(ctypes.byref(cfg), ctypes.c_int64(first), ctypes.c_int64(n),
                                len1.ctypes.data_as(p32), len2.ctypes.data_as(p32),
                                ref_off.ctypes.data_as(p64), qer_off.ctypes.data_as(p64),
                                ref.ctypes.data_as(pu8), qer.ctypes.data_as(pu8), nthreads)
        if rc != 0:
            raise RuntimeError("tal_synth_fill failed")
    pairs = new_pairs(n)
    pairs["idr"] = ref_off.astype(np.int32)
    pairs["idq"] = qer_off.astype(np.int32)
    pairs["id"] = np.arange(first, first + n, dtype=np.int64).astype(np.int32)
    pairs["len1"] = len1
    pairs["len2"] = len2
    pairs["h0"] = h0
    return Batch(pairs=pairs, ref=ref, qer=qer, w=w, workload=wl)


__all__ = ["Workload", "WORKLOADS", "C1", "C1_8", "C2", "C3", "C4", "Batch", "generate",
           "SEQPAIR_DTYPE"]
