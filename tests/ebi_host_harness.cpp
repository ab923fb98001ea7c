// Host build of the EBI device code for the CPU tests: csrc/ebi.cuh's per-cell HRSOLVER
// state machine (start, then one Backward-Euler iteration per call) with the mechanism's
// generated HRRATES, HRG1-4 and HRPRODLOSS (gen/<mech>_ebi.cu), compiled by g++ with
// tests/cuda_host_shim.h and run as cmaqchem_ebi_solve_device runs a lane (k_ebi_solve):
// cells in groups of 32 side by side in a warp's workspace block.  Built with
// AddressSanitizer and UndefinedBehaviorSanitizer by tests/test_ebi_host.py.
//
//   ebi_host_harness <in> <out> ncell tstep_sec
//   in:  yc [NSPEC][ncell] (mechanism order), rki [NRXNS][ncell] (doubles)
//   out: yc [NSPEC][ncell] (doubles), status, iterations [ncell] (int32 each)
#include <stdio.h>
#include <stdlib.h>

#define EBI_CELL_ONLY
#include "../cmaq_gb300/csrc/ebi.cuh"
#include MECH_HEADER

using M = MECH_NS::Traits;

int main(int argc, char** argv)
{
    if (argc != 5) return 2;
    const long long n = atoll(argv[3]);
    const int tstep_sec = atoi(argv[4]);
    if (n <= 0 || tstep_sec <= 0) return 2;
    const size_t ny = (size_t)M::NSPEC * n, nr = (size_t)M::NRXNS * n;
    double* yc = (double*)malloc(sizeof(double) * ny);
    double* rki = (double*)malloc(sizeof(double) * nr);
    FILE* fi = fopen(argv[1], "rb");
    if (!fi || fread(yc, sizeof(double), ny, fi) != ny || fread(rki, sizeof(double), nr, fi) != nr) return 3;
    fclose(fi);
    int n_ebi_steps = 0;
    double tmstep = 0.0;
    ebi::steps_for(tstep_sec, M::EBI_DELTAT, &n_ebi_steps, &tmstep);
    double* ws = (double*)malloc(sizeof(double) * (size_t)M::WS_ELEMS * 32);
    int* st = (int*)calloc((size_t)2 * n, sizeof(int));
    for (long long c = 0; c < n; ++c) {
        double* w = ws + c % 32;
        for (int i = 0; i < M::NSPEC; ++i) w[(M::EBI_OFF_YC + i) * 32] = yc[(size_t)i * n + c];
        for (int r = 0; r < M::NRXNS; ++r) w[(M::OFF_RKI + r) * 32] = rki[(size_t)r * n + c];
        ebi::State s;
        ebi::start<M>(w, s, n_ebi_steps, tmstep);
        while (!s.done) ebi::iterate<M>(w, s, 10000000);
        for (int i = 0; i < M::NSPEC; ++i) yc[(size_t)i * n + c] = w[(M::EBI_OFF_YC + i) * 32];
        st[c] = s.status;
        st[n + c] = s.total_iter;
    }
    FILE* fo = fopen(argv[2], "wb");
    if (!fo) return 4;
    fwrite(yc, sizeof(double), ny, fo);
    fwrite(st, sizeof(int), (size_t)2 * n, fo);
    fclose(fo);
    free(yc);
    free(rki);
    free(ws);
    free(st);
    return 0;
}
