// Host build of the KMT2 device code (cmaq_gb300/csrc/kmt2.cuh) for the CPU tests.
//
// Runs the kernels' cell queue serially: lanes 0 .. nlanes-1, each with its slice of the
// workspace (a warp's 32 lanes side by side, as on the device), take cells in lane order
// from a counter, and every pass of
// the loop advances each busy lane by one Rodas3 attempt (kmt2::kq_advance), as one pass
// of k_kmt2_queue / k_aqchem_queue (csrc/kmt2.cu) does for a warp.  Built with
// AddressSanitizer by tests/test_kmt2_host.py, so every workspace and array access of the
// device code is bounds-checked for the sizes the test runs.
//
//   kmt2_host_harness <in> <out> ncell nlanes
//   in:  params [NPARAM][ncell], var_mix [NVAR][ncell]          (doubles)
//   out: var_out [NVAR][ncell], fix_out [NFIX][ncell] (doubles), stats [NSTAT][ncell] (int32)
//
//   kmt2_host_harness aqchem <in> <out> ncell nlanes naer       (the whole AQCHEM)
//   in:  params [NPARAM][ncell], gas [29][ncell], aerosol [naer*3][ncell], factors [16] (doubles),
//        aer_index [31] (int32)
//   out: gas, aerosol, gas_wdep, aer_wdep, out [10][ncell] (doubles), stats [NSTAT][ncell] (int32)
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "../cmaq_gb300/csrc/kmt2.cuh"

// lane l's workspace: warp l / 32's block, column l % 32 (csrc/kmt2.cu)
static double* lane_ws(double* ws, long long l)
{
    return ws + (l / 32) * (kmt2::KQ_S * kmt2::WS_ELEMS) + l % 32;
}

// the workspace of nlanes lanes: whole warps
static double* alloc_ws(long long nlanes)
{
    return (double*)malloc(sizeof(double) * kmt2::KQ_S * kmt2::WS_ELEMS * ((nlanes + 31) / 32));
}

struct Slot {   // a lane between attempts
    kmt2::Cell c;
    kmt2::Lane L;
    long long st[kmt2::NSTAT];
    long long cell = -1;
};

// The kernels' loop: begin(q, l) starts q.cell in lane l's slice, done(q, l) writes its
// outputs when kq_advance has ended it.
template <class Begin, class Done>
static void run_queue(long long ncell, long long nlanes, double* ws, Begin begin, Done done)
{
    std::vector<Slot> lanes((size_t)nlanes);
    long long next = 0;
    for (;;) {
        bool busy = false;
        for (long long l = 0; l < nlanes; ++l) {
            Slot& q = lanes[(size_t)l];
            if (q.cell < 0 && next < ncell) {
                q.cell = next++;
                begin(q, l);
            }
            busy = busy || q.cell >= 0;
        }
        if (!busy) break;
        for (long long l = 0; l < nlanes; ++l) {
            Slot& q = lanes[(size_t)l];
            if (q.cell >= 0 && kmt2::kq_advance(q.c, q.L, lane_ws(ws, l), q.st)) {
                done(q, l);
                q.cell = -1;
            }
        }
    }
}

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
    double* ws = alloc_ws(nlanes);
    int nfail = 0;
    const long long n = ncell;
    run_queue(
        ncell, nlanes, ws,
        [&](Slot& q, long long l) {
            const long long c = q.cell;
            double* w = lane_ws(ws, l);
            kmt2::kq_aq_map(params + c, gas + c, aer + c, naer, aidx, fac, n, w);
            kmt2::kq_begin(q.c, q.L, params + c, n, w + kmt2::W_YNEW * kmt2::KQ_S, kmt2::KQ_S, gas[kmt2::KG_HO * n + c],
                           w, q.st);
        },
        [&](Slot& q, long long l) {
            const long long c = q.cell;
            nfail += kmt2::kq_aq_finish(q.c, q.L.ierr, q.st, params + c, gas + c, aer + c, naer, aidx, fac, gwd + c,
                                        awd + c, out + c, st + c, n, lane_ws(ws, l));
        });
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
    double* ws = alloc_ws(nlanes);
    const double* params = in;
    const double* vmix = in + (size_t)kmt2::NPARAM * ncell;
    int nfail = 0;
    const long long n = ncell;
    run_queue(
        ncell, nlanes, ws,
        [&](Slot& q, long long l) {
            const long long c = q.cell;
            kmt2::kq_begin(q.c, q.L, params + c, n, vmix + c, n, params[kmt2::P_HO * n + c], lane_ws(ws, l), q.st);
        },
        [&](Slot& q, long long l) {
            const long long c = q.cell;
            const double* y = lane_ws(ws, l) + kmt2::W_Y * kmt2::KQ_S;
            const double* f = lane_ws(ws, l) + kmt2::W_F * kmt2::KQ_S;
            const bool nan = q.L.ierr <= -101;   // failed set-up: no state to return
            for (int i = 0; i < kmt2::NVAR; ++i) vout[i * n + c] = nan ? (double)NAN : y[i * kmt2::KQ_S];
            for (int i = 0; i < kmt2::NFIX; ++i) fout[i * n + c] = nan ? (double)NAN : f[i * kmt2::KQ_S];
            for (int i = 0; i < kmt2::NSTAT; ++i) st[i * n + c] = (int)q.st[i];
            nfail += q.L.ierr == 1 ? 0 : 1;
        });
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
