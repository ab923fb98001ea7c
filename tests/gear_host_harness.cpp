// Host build of the SMVGEAR device code for the CPU tests: csrc/gear.cuh's per-cell state
// machine (gear::start, then gear::advance and gear::evaluate until the cell is done) with
// the generated f, Jacobian (PDERIV) and LU routines of gen/<mech>_rates.cu, _glu*.cu and
// _solve0.cu, compiled by g++ with tests/cuda_host_shim.h and run as
// cmaqchem_gear_solve_device runs a lane (k_gear, solver level): cells in groups of 32 side
// by side in a warp's workspace block.  Built with AddressSanitizer and
// UndefinedBehaviorSanitizer by tests/test_gear_host.py.
//
//   gear_host_harness <in> <out> ncell chemstep_min rtol max_atol min_atol conc_floor
//   in:  y [NSPEC][ncell] (solver order), rk [NRXNS][ncell] (doubles), night [ncell] (uint8)
//   out: y [NSPEC][ncell] (doubles), stats [ncell][8] (int32: nsteps, ncfail, nefail,
//        npderiv, nsubfun, nnewt, maxord, status)
#include <stdio.h>
#include <stdlib.h>

#define GEAR_CELL_ONLY
#include "../cmaq_gb300/csrc/gear.cuh"
#include MECH_HEADER

using M = MECH_NS::Traits;

int main(int argc, char** argv)
{
    if (argc != 9) return 2;
    const long long n = atoll(argv[3]);
    const double chemstep = atof(argv[4]), rtol = atof(argv[5]);
    const float max_atol = (float)atof(argv[6]), min_atol = (float)atof(argv[7]), floor_ = (float)atof(argv[8]);
    if (n <= 0 || !(chemstep > 0.0)) return 2;
    const size_t ny = (size_t)M::NSPEC * n, nr = (size_t)M::NRXNS * n;
    double* y = (double*)malloc(sizeof(double) * ny);
    double* rk = (double*)malloc(sizeof(double) * nr);
    unsigned char* night = (unsigned char*)malloc((size_t)n);
    FILE* fi = fopen(argv[1], "rb");
    if (!fi || fread(y, sizeof(double), ny, fi) != ny || fread(rk, sizeof(double), nr, fi) != nr ||
        fread(night, 1, (size_t)n, fi) != (size_t)n)
        return 3;
    fclose(fi);
    gear::Coef K;
    gear::coefficients(rtol, max_atol, min_atol, floor_, 100000, &K);
    double* ws = (double*)malloc(sizeof(double) * (size_t)M::GEAR_WS_ELEMS * 32);
    int* st = (int*)calloc((size_t)8 * n, sizeof(int));
    for (long long c = 0; c < n; ++c) {
        double* w = ws + c % 32;
        for (int i = 0; i < M::NSPEC; ++i) w[(M::GEAR_CNEW + i) * 32] = y[(size_t)i * n + c];
        for (int r = 0; r < M::NRXNS; ++r) w[(M::OFF_RKI + r) * 32] = rk[(size_t)r * n + c];
        gear::State s;
        gear::start<M, 32, false>(s, w, night[c] == 0, &K, false);
        while (gear::advance<M, 32, false>(w, s, &K, chemstep) != gear::DONE) gear::evaluate<M, 32, false>(w, s, true);
        for (int i = 0; i < M::NSPEC; ++i) y[(size_t)i * n + c] = w[(M::GEAR_CNEW + i) * 32];
        int* o = st + (size_t)8 * c;
        o[0] = s.st.nsteps; o[1] = s.st.ncfail; o[2] = s.st.nefail; o[3] = s.st.npderiv;
        o[4] = s.st.nsubfun; o[5] = s.st.nnewt; o[6] = s.st.maxord; o[7] = s.st.status;
    }
    FILE* fo = fopen(argv[2], "wb");
    if (!fo) return 4;
    fwrite(y, sizeof(double), ny, fo);
    fwrite(st, sizeof(int), (size_t)8 * n, fo);
    fclose(fo);
    free(y);
    free(rk);
    free(night);
    free(ws);
    free(st);
    return 0;
}
