// Host build of the HETCHEM_RATES device code (cmaq_gb300/csrc/hetchem.cuh) for the CPU
// tests: the kernel's per-cell function over every cell, serially, on the same
// [row][cell] arrays.  Built with AddressSanitizer and UndefinedBehaviorSanitizer by
// tests/test_hetchem_host.py, once per mechanism (HET_NS / HET_GEN as hetchem.cuh takes
// them; CB6r5 without).
//
//   hetchem_host_harness <in> <out> ncell
//   in:  ae [NAE][ncell], ta, pres, qv, dens [ncell]   (float32)
//   out: khetero [ncell][NHET]                         (float64)
#include <stdio.h>
#include <stdlib.h>

#include "../cmaq_gb300/csrc/hetchem.cuh"

namespace HET_NS {
static const HetTables host_tables = HET_TABLES_INIT;
}

int main(int argc, char** argv)
{
    if (argc != 4) return 2;
    const long long ncell = atoll(argv[3]);
    if (ncell <= 0) return 2;
    const size_t nin = (size_t)(HET_NS::NAE + 4) * ncell;
    float* in = (float*)malloc(sizeof(float) * nin);
    FILE* fi = fopen(argv[1], "rb");
    if (!fi || fread(in, sizeof(float), nin, fi) != nin) return 3;
    fclose(fi);
    const float* ae = in;
    const float* met = in + (size_t)HET_NS::NAE * ncell;
    double* k = (double*)malloc(sizeof(double) * HET_NS::NHET * ncell);
    for (long long c = 0; c < ncell; ++c)
        HET_NS::het_cell(HET_NS::host_tables, ae + c, ncell, met[c], met[ncell + c], met[2 * ncell + c], met[3 * ncell + c],
                      k + c * HET_NS::NHET);
    FILE* fo = fopen(argv[2], "wb");
    if (!fo) return 4;
    fwrite(k, sizeof(double), (size_t)HET_NS::NHET * ncell, fo);
    fclose(fo);
    free(in);
    free(k);
    return 0;
}
