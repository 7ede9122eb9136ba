"""GB300 banded Smith-Waterman seed extension (TAL BandedPairWiseSW drop-in).

The compute path is the CUDA library lib/libtal_bsw.so (csrc/), reached through
the C ABI declared in include/tal_bsw.h; this package is its Python front end
plus the seeded synthetic workloads used by the benchmark and the tests."""
from .seqpair import SEQPAIR_DTYPE, SEQPAIR_FIELDS, OUTPUT_FIELDS, new_pairs, outputs  # noqa: F401
from .api import BandedPairWiseSW, BswServer, TalBswError, AUTO, BITS8, BITS16  # noqa: F401
from ._lib import PKG_DIR, LIB_DIR, CORE_LIB, SYNTH_LIB  # noqa: F401
