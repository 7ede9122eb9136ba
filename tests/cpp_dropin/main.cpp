// A caller written against the reference's bandedSWA.h interface (as
// benchmarks/bench-bsw.cpp:213-258 calls it), compiled against the GB300
// drop-in header instead.  Test program: reads a batch from a binary file,
// scores it with getScores8 / getScores16 / scalarBandedSWAWrapper, writes
// the scored SeqPair records back.
//   input:  int64 n, int32 w, int32 mode (8, 16, or 0 = scalar wrapper),
//           int32 params[8] (o_del e_del o_ins e_ins zdrop end_bonus a b),
//           SeqPair[n], int64 nref, ref bytes, int64 nqer, query bytes
//   output: SeqPair[n], then uint64 SW_cells
#include <stdio.h>
#include <stdlib.h>

#include <vector>

#include "bandedSWA_gb300.h"

// bench-bsw.cpp:56-64: a on the diagonal, -b off it, ambig in row/column 4
static void fill_scmat(int a, int b, int ambig, int8_t mat[25]) {
    int k = 0;
    for (int i = 0; i < 4; ++i) {
        for (int j = 0; j < 4; ++j) mat[k++] = i == j ? a : -b;
        mat[k++] = ambig;
    }
    for (int j = 0; j < 5; ++j) mat[k++] = ambig;
}

int main(int argc, char **argv) {
    if (argc != 3) return 2;
    FILE *f = fopen(argv[1], "rb");
    if (!f) return 2;
    int64_t n = 0, nr = 0, nq = 0;
    int32_t w = 0, mode = 0, P[8];
    if (fread(&n, 8, 1, f) != 1 || fread(&w, 4, 1, f) != 1 || fread(&mode, 4, 1, f) != 1 ||
        fread(P, 4, 8, f) != 8)
        return 2;
    std::vector<SeqPair> pairs(n);
    if (fread(pairs.data(), sizeof(SeqPair), n, f) != (size_t)n || fread(&nr, 8, 1, f) != 1) return 2;
    std::vector<uint8_t> ref(nr);
    if (fread(ref.data(), 1, nr, f) != (size_t)nr || fread(&nq, 8, 1, f) != 1) return 2;
    std::vector<uint8_t> qer(nq);
    if (fread(qer.data(), 1, nq, f) != (size_t)nq) return 2;
    fclose(f);
    int8_t mat[25];
    fill_scmat(P[6], P[7], -1, mat);
    BandedPairWiseSW bsw(P[0], P[1], P[2], P[3], P[4], P[5], mat, (int8_t)P[6], (int8_t)P[7], 1);
    if (mode == 16) bsw.getScores16(pairs.data(), ref.data(), qer.data(), (int32_t)n, 1, w);
    else if (mode == 8) bsw.getScores8(pairs.data(), ref.data(), qer.data(), (int32_t)n, 1, w);
    else bsw.scalarBandedSWAWrapper(pairs.data(), ref.data(), qer.data(), (int)n, 1, w);
    FILE *o = fopen(argv[2], "wb");
    if (!o) return 2;
    fwrite(pairs.data(), sizeof(SeqPair), n, o);
    fwrite(&bsw.SW_cells, 8, 1, o);
    fclose(o);
    return 0;
}
