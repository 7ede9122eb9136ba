// Test infrastructure only: a C entry point around the reference's own DP
// chaining (src/chaining/parallel_chaining_32_bit.h, dp_chain), compiled from
// the read-only reference tree by oracle/build_ref.sh into oracle/_ref/.  Used
// to pin the oracle (oracle/chain_oracle.cpp) and to generate golden fixtures;
// never linked into the product library.
//
// Driven the way benchmarks/bench-dp-chaining.cpp drives it: one dp_chain
// built from its eight tunables, then per read the structure-of-arrays copy
// (create_SoA_Anchors_32_bit) and mm_dp_vectorized(n, anchors, r, q, l, f, p,
// v, dr, dq, NULL, NULL), with f, p and v allocated 16 entries past their
// start as the driver does (the vector loop reads below a read's first anchor).
// The header uses the fixed-width integer types without including their
// header; the reference's driver includes it (through <x86intrin.h> and the
// standard headers) first.
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <x86intrin.h>

#include "parallel_chaining_32_bit.h"

extern "C" {

int ref_chain_run(int max_dist_x, int max_dist_y, int bw, int max_skip, int max_iter,
                  float gap_scale, int is_cdna, int n_segs, const void *anchors,
                  const int64_t *offsets, int32_t n_reads, int32_t dr, int32_t dq, uint32_t *f,
                  int32_t *p, int32_t *v) {
    dp_chain obj(max_dist_x, max_dist_y, bw, max_skip, max_iter, gap_scale, is_cdna, n_segs);
    const anchor_t *all = static_cast<const anchor_t *>(anchors);
    for (int32_t k = 0; k < n_reads; k++) {
        const int64_t o = offsets[k], n = offsets[k + 1] - offsets[k];
        if (n <= 0) continue;
        std::vector<anchor_t> anc(all + o, all + o + n);
        uint32_t *fb = (uint32_t *)calloc((size_t)n + 16, sizeof(uint32_t));
        int32_t *pb = (int32_t *)calloc((size_t)n + 16, sizeof(int32_t));
        int32_t *vb = (int32_t *)calloc((size_t)n + 16, sizeof(int32_t));
        uint32_t *fr = fb + 16;
        int32_t *pr = pb + 16, *vr = vb + 16;
        uint32_t *ar, *aq, *al;
        create_SoA_Anchors_32_bit(&anc[0], (uint32_t)n, ar, aq, al);
        obj.mm_dp_vectorized(n, &anc[0], ar, aq, al, fr, pr, vr, dr, dq, NULL, NULL);
        memcpy(f + o, fr, sizeof(uint32_t) * (size_t)n);
        memcpy(p + o, pr, sizeof(int32_t) * (size_t)n);
        memcpy(v + o, vr, sizeof(int32_t) * (size_t)n);
        free(ar - 16);
        free(aq - 16);
        free(al - 16);
        free(fb);
        free(pb);
        free(vb);
    }
    return 0;
}

}  // extern "C"
