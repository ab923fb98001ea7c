// Host build of the ROS3 device code for the CPU tests: csrc/ros3.cuh's per-cell
// integration (rbsolver.F's time loop) with the generated mechanism routines of
// gen/<mech>_rates.cu, _lu*.cu and _solve*.cu, compiled by g++ with tests/cuda_host_shim.h
// and run as cmaqchem_ros3_solve_device runs a warp: cells in groups of 32 side by side in
// a warp's workspace block ([element][32 lanes]), the night reaction list only when every
// cell of the group is dark.  Built with AddressSanitizer and UndefinedBehaviorSanitizer
// by tests/test_ros3_host.py, so every workspace index of the generated code is checked.
//
//   ros3_host_harness <in> <out> ncell chemstep_min rtol atol
//   in:  y [ISCHAN][ncell], rki [NRXNS][ncell] (doubles), night [ncell] (uint8)
//   out: y [ISCHAN][ncell] (doubles), nsteps, nfails, status [ncell] (int32 each)
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../cmaq_gb300/csrc/ros3.cuh"
#include MECH_HEADER

using M = MECH_NS::Traits;

int main(int argc, char** argv)
{
    if (argc != 7) return 2;
    const long long n = atoll(argv[3]);
    const double chemstep = atof(argv[4]), rtol = atof(argv[5]), atol = atof(argv[6]);
    if (n <= 0 || !(chemstep > 0.0)) return 2;
    const size_t ny = (size_t)M::ISCHAN * n, nr = (size_t)M::NRXNS * n;
    double* y = (double*)malloc(sizeof(double) * ny);
    double* rki = (double*)malloc(sizeof(double) * nr);
    unsigned char* night = (unsigned char*)malloc((size_t)n);
    FILE* fi = fopen(argv[1], "rb");
    if (!fi || fread(y, sizeof(double), ny, fi) != ny || fread(rki, sizeof(double), nr, fi) != nr ||
        fread(night, 1, (size_t)n, fi) != (size_t)n)
        return 3;
    fclose(fi);
    const size_t block = (size_t)M::WS_ELEMS * 32;   // one warp's workspace
    double* ws = (double*)malloc(sizeof(double) * block);
    int* st = (int*)calloc((size_t)3 * n, sizeof(int));
    // RNSPEC = 1.0 / FLOAT(N_SPEC) in REAL(4), as the library sets it
    const ros3::Tol tol{rtol, atol, (double)(1.0f / (float)M::NSPEC), ros3::DTMIN};
    for (long long base = 0; base < n; base += 32) {
        const long long m = n - base < 32 ? n - base : 32;
        bool dark = true;
        for (long long l = 0; l < m; ++l) dark = dark && night[base + l] != 0;
        for (long long l = 0; l < m; ++l) {
            const long long c = base + l;
            double* w = ws + l;
            for (int i = 0; i < M::ISCHAN; ++i) w[(M::OFF_Y + i) * 32] = y[(size_t)i * n + c];
            for (int r = 0; r < M::NRXNS; ++r) w[(M::OFF_RKI + r) * 32] = rki[(size_t)r * n + c];
            const ros3::CellStats s = ros3::integrate<M>(w, chemstep, tol, dark, 100000);
            for (int i = 0; i < M::ISCHAN; ++i) y[(size_t)i * n + c] = w[(M::OFF_Y + i) * 32];
            st[c] = s.nsteps;
            st[n + c] = s.nfails;
            st[2 * n + c] = s.status;
        }
    }
    FILE* fo = fopen(argv[2], "wb");
    if (!fo) return 4;
    fwrite(y, sizeof(double), ny, fo);
    fwrite(st, sizeof(int), (size_t)3 * n, fo);
    fclose(fo);
    free(y);
    free(rki);
    free(night);
    free(ws);
    free(st);
    printf("%d\n", M::WS_ELEMS);
    return 0;
}
