// Host build of the KMT2 device code (cmaq_gb300/csrc/kmt2.cuh) for the CPU tests.
//
// Runs the kernel's loop, lane by lane, over the cells: lane l integrates cells
// l, l + nlanes, ... in its slice of the lane-interleaved workspace, exactly the
// indexing of k_kmt2_cells (csrc/kmt2.cu), serially.  Built with AddressSanitizer by
// tests/test_kmt2_host.py, so every workspace and array access of the device code is
// bounds-checked for the sizes the test runs.
//
//   kmt2_host_harness <in> <out> ncell nlanes
//   in:  params [NPARAM][ncell], var_mix [NVAR][ncell]          (doubles)
//   out: var_out [NVAR][ncell], fix_out [NFIX][ncell] (doubles), stats [NSTAT][ncell] (int32)
//
//   kmt2_host_harness aqchem <in> <out> ncell nlanes naer       (the whole AQCHEM, kq_aqchem_cell)
//   in:  params [NPARAM][ncell], gas [29][ncell], aerosol [naer*3][ncell], factors [16] (doubles),
//        aer_index [31] (int32)
//   out: gas, aerosol, gas_wdep, aer_wdep, out [10][ncell] (doubles), stats [NSTAT][ncell] (int32)
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../cmaq_gb300/csrc/kmt2.cuh"

static int run_aqchem(int argc, char** argv)
{
    if (argc != 7) return 2;
    const long long ncell = atoll(argv[4]), nlanes = atoll(argv[5]);
    const int naer = atoi(argv[6]);
    if (ncell <= 0 || nlanes <= 0 || naer <= 0) return 2;
    const size_t ng = (size_t)kmt2::KG_NGAS * ncell, na = (size_t)naer * 3 * ncell;
    const size_t nd = (size_t)kmt2::NPARAM * ncell + ng + na + kmt2::KF_N;
    double* in = (double*)malloc(sizeof(double) * nd);
    int aidx[kmt2::KA_NIDX];
    FILE* fi = fopen(argv[2], "rb");
    if (!fi || fread(in, sizeof(double), nd, fi) != nd || fread(aidx, sizeof(int), kmt2::KA_NIDX, fi) != kmt2::KA_NIDX)
        return 3;
    fclose(fi);
    const double* params = in;
    double* gas = in + (size_t)kmt2::NPARAM * ncell;
    double* aer = gas + ng;
    const double* fac = aer + na;
    double* gwd = (double*)calloc(ng, sizeof(double));
    double* awd = (double*)calloc(na, sizeof(double));
    double* out = (double*)calloc((size_t)kmt2::KO_N * ncell, sizeof(double));
    int* st = (int*)calloc((size_t)kmt2::NSTAT * ncell, sizeof(int));
    double* ws = (double*)malloc(sizeof(double) * kmt2::WS_ELEMS * nlanes);
    int nfail = 0;
    for (long long lane = 0; lane < nlanes; ++lane)
        for (long long c = lane; c < ncell; c += nlanes)
            nfail += kmt2::kq_aqchem_cell(params + c, gas + c, aer + c, naer, aidx, fac, gwd + c, awd + c, out + c,
                                          st + c, ncell, ws + lane, nlanes);
    FILE* fo = fopen(argv[3], "wb");
    if (!fo) return 4;
    fwrite(gas, sizeof(double), ng, fo);
    fwrite(aer, sizeof(double), na, fo);
    fwrite(gwd, sizeof(double), ng, fo);
    fwrite(awd, sizeof(double), na, fo);
    fwrite(out, sizeof(double), (size_t)kmt2::KO_N * ncell, fo);
    fwrite(st, sizeof(int), (size_t)kmt2::NSTAT * ncell, fo);
    fclose(fo);
    free(in);
    free(gwd);
    free(awd);
    free(out);
    free(st);
    free(ws);
    printf("%d %d\n", nfail, kmt2::WS_ELEMS);
    return 0;
}

int main(int argc, char** argv)
{
    if (argc > 1 && strcmp(argv[1], "aqchem") == 0) return run_aqchem(argc, argv);
    if (argc != 5) return 2;
    const long long ncell = atoll(argv[3]), nlanes = atoll(argv[4]);
    if (ncell <= 0 || nlanes <= 0) return 2;
    const size_t nin = (size_t)(kmt2::NPARAM + kmt2::NVAR) * ncell;
    double* in = (double*)malloc(sizeof(double) * nin);
    FILE* fi = fopen(argv[1], "rb");
    if (!fi || fread(in, sizeof(double), nin, fi) != nin) return 3;
    fclose(fi);
    double* vout = (double*)calloc((size_t)kmt2::NVAR * ncell, sizeof(double));
    double* fout = (double*)calloc((size_t)kmt2::NFIX * ncell, sizeof(double));
    int* st = (int*)calloc((size_t)kmt2::NSTAT * ncell, sizeof(int));
    double* ws = (double*)malloc(sizeof(double) * kmt2::WS_ELEMS * nlanes);
    const double* params = in;
    const double* vmix = in + (size_t)kmt2::NPARAM * ncell;
    int nfail = 0;
    for (long long lane = 0; lane < nlanes; ++lane)
        for (long long c = lane; c < ncell; c += nlanes)
            nfail += kmt2::kq_cell(params + c, vmix + c, vout + c, fout + c, st + c, ncell, ws + lane, nlanes);
    FILE* fo = fopen(argv[2], "wb");
    if (!fo) return 4;
    fwrite(vout, sizeof(double), (size_t)kmt2::NVAR * ncell, fo);
    fwrite(fout, sizeof(double), (size_t)kmt2::NFIX * ncell, fo);
    fwrite(st, sizeof(int), (size_t)kmt2::NSTAT * ncell, fo);
    fclose(fo);
    free(in);
    free(vout);
    free(fout);
    free(st);
    free(ws);
    printf("%d %d\n", nfail, kmt2::WS_ELEMS);
    return 0;
}
