#!/usr/bin/env bash
# Builds the reference's own banded Smith-Waterman (bandedSWA.cpp) from the
# read-only reference tree (its root in TAL_REFERENCE_ROOT) into oracle/_ref/,
# for pinning the oracle and for generating golden fixtures.  Test
# infrastructure only.
#
# The reference header includes "macro.h", which the reference tree does not
# ship; an empty stub stands in for it.  x86-64 only: the kernels under test are
# the AVX-512BW (and AVX2) paths.  On any other host this script does nothing.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
# the reference tree's root comes from the environment only
if [ -z "${TAL_REFERENCE_ROOT:-}" ]; then
  echo "build_ref: TAL_REFERENCE_ROOT is not set; skipping" >&2
  exit 0
fi
REF_BSW="$TAL_REFERENCE_ROOT/src/alignment/BSW"
OUT="$HERE/_ref"
if [ ! -f "$REF_BSW/bandedSWA.cpp" ]; then
  echo "build_ref: reference sources not present; skipping" >&2
  exit 0
fi
case "$(uname -m)" in
  x86_64) ;;
  *) echo "build_ref: reference SIMD paths are x86-only; skipping" >&2; exit 0 ;;
esac
mkdir -p "$OUT/stub"
: > "$OUT/stub/macro.h"
build() {  # $1 = isa flag, $2 = suffix
  g++ -O2 -fPIC -shared $1 -w -I"$OUT/stub" -I"$REF_BSW" \
      "$REF_BSW/bandedSWA.cpp" "$HERE/ref_shim.cpp" -o "$OUT/libbsw_ref_$2.so"
}
if grep -q avx512bw /proc/cpuinfo; then
  build -mavx512bw avx512 &
fi
build -mavx2 avx2 &

# The unbanded Smith-Waterman classes (src/alignment/Smith-Waterman).  Their
# header defines its own __rdtsc, which clashes with the compiler's: each
# reference source is compiled through a one-line wrapper that includes
# <immintrin.h> first and renames the header's copy.
REF_SW="$TAL_REFERENCE_ROOT/src/alignment/Smith-Waterman"
if [ -f "$REF_SW/PairWiseSW_16.cpp" ] && grep -q avx512bw /proc/cpuinfo; then
  mkdir -p "$OUT/sw_wrap"
  for f in PairWiseSW PairWiseSW_8 PairWiseSW_16 PairWiseSW_32; do
    printf '#include <immintrin.h>\n#define __rdtsc tal_ref_rdtsc\n#include "%s/%s.cpp"\n' \
      "$REF_SW" "$f" > "$OUT/sw_wrap/$f.cpp"
  done
  g++ -O2 -fPIC -shared -mavx512bw -fopenmp -w -I"$REF_SW" "$OUT"/sw_wrap/*.cpp \
      "$HERE/ref_sw_shim.cpp" -o "$OUT/libsw_ref_avx512.so" &
fi

# The DP chaining (src/chaining/parallel_chaining_32_bit.h), header only: the
# AVX-512 path (the one benchmarks/bench-dp-chaining.cpp runs on an AVX-512
# host), the same under the reference Makefile's -Ofast (fast-math may
# reassociate the scalar path's double product), and the AVX2 path.
REF_CH="$TAL_REFERENCE_ROOT/src/chaining"
if [ -f "$REF_CH/parallel_chaining_32_bit.h" ]; then
  chain() {  # $1 = flags, $2 = suffix
    g++ -fPIC -shared $1 -w -I"$REF_CH" "$HERE/ref_chain_shim.cpp" -o "$OUT/libchain_ref_$2.so"
  }
  if grep -q avx512cd /proc/cpuinfo; then
    chain "-O2 -mavx512f -mavx512bw -mavx512cd -mavx512vl" avx512 &
    chain "-Ofast -mavx512f -mavx512bw -mavx512cd -mavx512vl" avx512_ofast &
  fi
  chain "-O2 -mavx2" avx2 &
fi
wait
ls "$OUT"/*.so
