// Generated by cmaq_gb300.mechgen.generate from CCTM/src/MECHS/cb6r5_ae7_aq/RXNS_DATA_MODULE.F90
// and RXNS_FUNC_MODULE.F90 (sha256/16 4242f44b2527a299).  Do not edit.
#include "cb6r5_ae7_aq_mech.cuh"
#include <math.h>
namespace mech_cb6r5_ae7_aq {
__device__ __noinline__ void solve_s1_0_0(double* __restrict__ ws, int rhs)
{
    const double* __restrict__ lu = ws + 2426;
    const double* __restrict__ vd = ws + 4116;
    double* __restrict__ b = ws + rhs;
    (void)vd;
    {
      double x = b[0];
      b[0] = x;
    }
    {
      double x = b[1];
      x = fma(-CHEM_LDLU(lu + 1), b[0], x);
      b[1] = x;
    }
    {
      double x = b[2];
      b[2] = x;
    }
    {
      double x = b[3];
      b[3] = x;
    }
    {
      double x = b[4];
      b[4] = x;
    }
    {
      double x = b[5];
      b[5] = x;
    }
    {
      double x = b[6];
      b[6] = x;
    }
    {
      double x = b[7];
      b[7] = x;
    }
    {
      double x = b[8];
      b[8] = x;
    }
    {
      double x = b[9];
      b[9] = x;
    }
    {
      double x = b[10];
      b[10] = x;
    }
    {
      double x = b[11];
      b[11] = x;
    }
    {
      double x = b[12];
      b[12] = x;
    }
    {
      double x = b[13];
      b[13] = x;
    }
    {
      double x = b[14];
      b[14] = x;
    }
    {
      double x = b[15];
      b[15] = x;
    }
    {
      double x = b[16];
      b[16] = x;
    }
    {
      double x = b[17];
      b[17] = x;
    }
    {
      double x = b[18];
      b[18] = x;
    }
    {
      double x = b[19];
      x = fma(-CHEM_LDLU(lu + 2), b[18], x);
      b[19] = x;
    }
    {
      double x = b[20];
      b[20] = x;
    }
    {
      double x = b[21];
      b[21] = x;
    }
    {
      double x = b[22];
      b[22] = x;
    }
    {
      double x = b[23];
      b[23] = x;
    }
    {
      double x = b[24];
      b[24] = x;
    }
    {
      double x = b[25];
      x = fma(-CHEM_LDLU(lu + 3), b[24], x);
      b[25] = x;
    }
    {
      double x = b[26];
      b[26] = x;
    }
    {
      double x = b[27];
      b[27] = x;
    }
    {
      double x = b[28];
      b[28] = x;
    }
    {
      double x = b[29];
      x = fma(-CHEM_LDLU(lu + 4), b[28], x);
      b[29] = x;
    }
    {
      double x = b[30];
      b[30] = x;
    }
    {
      double x = b[31];
      b[31] = x;
    }
    {
      double x = b[32];
      b[32] = x;
    }
    {
      double x = b[33];
      b[33] = x;
    }
    {
      double x = b[34];
      b[34] = x;
    }
    {
      double x = b[35];
      b[35] = x;
    }
    {
      double x = b[36];
      b[36] = x;
    }
    {
      double x = b[37];
      b[37] = x;
    }
    {
      double x = b[38];
      b[38] = x;
    }
    {
      double x = b[39];
      x = fma(-CHEM_LDLU(lu + 5), b[17], x);
      b[39] = x;
    }
    {
      double x = b[40];
      b[40] = x;
    }
    {
      double x = b[41];
      x = fma(-CHEM_LDLU(lu + 6), b[18], x);
      x = fma(-CHEM_LDLU(lu + 7), b[33], x);
      b[41] = x;
    }
    {
      double x = b[42];
      b[42] = x;
    }
    {
      double x = b[43];
      x = fma(-CHEM_LDLU(lu + 8), b[2], x);
      x = fma(-CHEM_LDLU(lu + 9), b[3], x);
      x = fma(-CHEM_LDLU(lu + 10), b[4], x);
      b[43] = x;
    }
    {
      double x = b[44];
      x = fma(-CHEM_LDLU(lu + 11), b[5], x);
      x = fma(-CHEM_LDLU(lu + 12), b[6], x);
      x = fma(-CHEM_LDLU(lu + 13), b[7], x);
      b[44] = x;
    }
    {
      double x = b[45];
      x = fma(-CHEM_LDLU(lu + 14), b[22], x);
      b[45] = x;
    }
    {
      double x = b[46];
      x = fma(-CHEM_LDLU(lu + 15), b[23], x);
      b[46] = x;
    }
    {
      double x = b[47];
      b[47] = x;
    }
    {
      double x = b[48];
      b[48] = x;
    }
    {
      double x = b[49];
      b[49] = x;
    }
    {
      double x = b[50];
      b[50] = x;
    }
    {
      double x = b[51];
      b[51] = x;
    }
    {
      double x = b[52];
      b[52] = x;
    }
    {
      double x = b[53];
      b[53] = x;
    }
    {
      double x = b[54];
      b[54] = x;
    }
    {
      double x = b[55];
      b[55] = x;
    }
    {
      double x = b[56];
      b[56] = x;
    }
    {
      double x = b[57];
      x = fma(-CHEM_LDLU(lu + 16), b[38], x);
      b[57] = x;
    }
    {
      double x = b[58];
      b[58] = x;
    }
    {
      double x = b[59];
      x = fma(-CHEM_LDLU(lu + 17), b[58], x);
      b[59] = x;
    }
    {
      double x = b[60];
      x = fma(-CHEM_LDLU(lu + 18), b[15], x);
      x = fma(-CHEM_LDLU(lu + 19), b[16], x);
      x = fma(-CHEM_LDLU(lu + 20), b[40], x);
      b[60] = x;
    }
    {
      double x = b[61];
      b[61] = x;
    }
    {
      double x = b[62];
      b[62] = x;
    }
    {
      double x = b[63];
      b[63] = x;
    }
    {
      double x = b[64];
      b[64] = x;
    }
    {
      double x = b[65];
      x = fma(-CHEM_LDLU(lu + 21), b[64], x);
      b[65] = x;
    }
    {
      double x = b[66];
      b[66] = x;
    }
    {
      double x = b[67];
      x = fma(-CHEM_LDLU(lu + 22), b[12], x);
      b[67] = x;
    }
    {
      double x = b[68];
      b[68] = x;
    }
    {
      double x = b[69];
      x = fma(-CHEM_LDLU(lu + 23), b[63], x);
      b[69] = x;
    }
    {
      double x = b[70];
      x = fma(-CHEM_LDLU(lu + 24), b[67], x);
      b[70] = x;
    }
    {
      double x = b[71];
      x = fma(-CHEM_LDLU(lu + 25), b[54], x);
      b[71] = x;
    }
    {
      double x = b[72];
      b[72] = x;
    }
    {
      double x = b[73];
      b[73] = x;
    }
    {
      double x = b[74];
      b[74] = x;
    }
    {
      double x = b[75];
      b[75] = x;
    }
    {
      double x = b[76];
      b[76] = x;
    }
    {
      double x = b[77];
      x = fma(-CHEM_LDLU(lu + 26), b[68], x);
      b[77] = x;
    }
    {
      double x = b[78];
      x = fma(-CHEM_LDLU(lu + 27), b[35], x);
      b[78] = x;
    }
    {
      double x = b[79];
      b[79] = x;
    }
    {
      double x = b[80];
      x = fma(-CHEM_LDLU(lu + 28), b[36], x);
      b[80] = x;
    }
    {
      double x = b[81];
      x = fma(-CHEM_LDLU(lu + 29), b[15], x);
      x = fma(-CHEM_LDLU(lu + 30), b[16], x);
      x = fma(-CHEM_LDLU(lu + 31), b[17], x);
      x = fma(-CHEM_LDLU(lu + 32), b[39], x);
      x = fma(-CHEM_LDLU(lu + 33), b[40], x);
      x = fma(-CHEM_LDLU(lu + 34), b[60], x);
      b[81] = x;
    }
    {
      double x = b[82];
      x = fma(-CHEM_LDLU(lu + 35), b[14], x);
      x = fma(-CHEM_LDLU(lu + 36), b[78], x);
      x = fma(-CHEM_LDLU(lu + 37), b[80], x);
      b[82] = x;
    }
    {
      double x = b[83];
      b[83] = x;
    }
    {
      double x = b[84];
      b[84] = x;
    }
    {
      double x = b[85];
      b[85] = x;
    }
    {
      double x = b[86];
      x = fma(-CHEM_LDLU(lu + 38), b[47], x);
      x = fma(-CHEM_LDLU(lu + 39), b[72], x);
      b[86] = x;
    }
    {
      double x = b[87];
      x = fma(-CHEM_LDLU(lu + 40), b[47], x);
      x = fma(-CHEM_LDLU(lu + 41), b[72], x);
      x = fma(-CHEM_LDLU(lu + 42), b[86], x);
      b[87] = x;
    }
    {
      double x = b[88];
      x = fma(-CHEM_LDLU(lu + 43), b[47], x);
      x = fma(-CHEM_LDLU(lu + 44), b[72], x);
      x = fma(-CHEM_LDLU(lu + 45), b[86], x);
      x = fma(-CHEM_LDLU(lu + 46), b[87], x);
      b[88] = x;
    }
    {
      double x = b[89];
      x = fma(-CHEM_LDLU(lu + 47), b[64], x);
      b[89] = x;
    }
    {
      double x = b[90];
      b[90] = x;
    }
    {
      double x = b[91];
      b[91] = x;
    }
    {
      double x = b[92];
      x = fma(-CHEM_LDLU(lu + 48), b[34], x);
      b[92] = x;
    }
    {
      double x = b[93];
      x = fma(-CHEM_LDLU(lu + 49), b[75], x);
      b[93] = x;
    }
    {
      double x = b[94];
      x = fma(-CHEM_LDLU(lu + 50), b[37], x);
      b[94] = x;
    }
    {
      double x = b[95];
      x = fma(-CHEM_LDLU(lu + 51), b[37], x);
      x = fma(-CHEM_LDLU(lu + 52), b[94], x);
      b[95] = x;
    }
    {
      double x = b[96];
      x = fma(-CHEM_LDLU(lu + 53), b[14], x);
      x = fma(-CHEM_LDLU(lu + 54), b[67], x);
      x = fma(-CHEM_LDLU(lu + 55), b[78], x);
      x = fma(-CHEM_LDLU(lu + 56), b[80], x);
      x = fma(-CHEM_LDLU(lu + 57), b[92], x);
      b[96] = x;
    }
    {
      double x = b[97];
      x = fma(-CHEM_LDLU(lu + 58), b[12], x);
      b[97] = x;
    }
    {
      double x = b[98];
      x = fma(-CHEM_LDLU(lu + 59), b[52], x);
      b[98] = x;
    }
    {
      double x = b[99];
      x = fma(-CHEM_LDLU(lu + 60), b[86], x);
      x = fma(-CHEM_LDLU(lu + 61), b[87], x);
      x = fma(-CHEM_LDLU(lu + 62), b[88], x);
      x = fma(-CHEM_LDLU(lu + 63), b[91], x);
      b[99] = x;
    }
    {
      double x = b[100];
      x = fma(-CHEM_LDLU(lu + 64), b[86], x);
      x = fma(-CHEM_LDLU(lu + 65), b[87], x);
      x = fma(-CHEM_LDLU(lu + 66), b[88], x);
      x = fma(-CHEM_LDLU(lu + 67), b[91], x);
      x = fma(-CHEM_LDLU(lu + 68), b[99], x);
      b[100] = x;
    }
    {
      double x = b[101];
      x = fma(-CHEM_LDLU(lu + 69), b[79], x);
      x = fma(-CHEM_LDLU(lu + 70), b[83], x);
      x = fma(-CHEM_LDLU(lu + 71), b[98], x);
      b[101] = x;
    }
    {
      double x = b[102];
      x = fma(-CHEM_LDLU(lu + 72), b[14], x);
      x = fma(-CHEM_LDLU(lu + 73), b[67], x);
      x = fma(-CHEM_LDLU(lu + 74), b[78], x);
      x = fma(-CHEM_LDLU(lu + 75), b[80], x);
      x = fma(-CHEM_LDLU(lu + 76), b[92], x);
      b[102] = x;
    }
    {
      double x = b[103];
      x = fma(-CHEM_LDLU(lu + 77), b[33], x);
      x = fma(-CHEM_LDLU(lu + 78), b[52], x);
      b[103] = x;
    }
    {
      double x = b[104];
      x = fma(-CHEM_LDLU(lu + 79), b[55], x);
      x = fma(-CHEM_LDLU(lu + 80), b[68], x);
      b[104] = x;
    }
    {
      double x = b[105];
      x = fma(-CHEM_LDLU(lu + 81), b[89], x);
      b[105] = x;
    }
    {
      double x = b[106];
      x = fma(-CHEM_LDLU(lu + 82), b[28], x);
      x = fma(-CHEM_LDLU(lu + 83), b[29], x);
      x = fma(-CHEM_LDLU(lu + 84), b[30], x);
      x = fma(-CHEM_LDLU(lu + 85), b[62], x);
      b[106] = x;
    }
    {
      double x = b[107];
      x = fma(-CHEM_LDLU(lu + 86), b[52], x);
      x = fma(-CHEM_LDLU(lu + 87), b[79], x);
      b[107] = x;
    }
    {
      double x = b[108];
      x = fma(-CHEM_LDLU(lu + 88), b[94], x);
      x = fma(-CHEM_LDLU(lu + 89), b[98], x);
      x = fma(-CHEM_LDLU(lu + 90), b[107], x);
      b[108] = x;
    }
    {
      double x = b[109];
      x = fma(-CHEM_LDLU(lu + 91), b[34], x);
      b[109] = x;
    }
    {
      double x = b[110];
      x = fma(-CHEM_LDLU(lu + 92), b[38], x);
      x = fma(-CHEM_LDLU(lu + 93), b[63], x);
      b[110] = x;
    }
    {
      double x = b[111];
      x = fma(-CHEM_LDLU(lu + 94), b[51], x);
      x = fma(-CHEM_LDLU(lu + 95), b[98], x);
      x = fma(-CHEM_LDLU(lu + 96), b[107], x);
      b[111] = x;
    }
    {
      double x = b[112];
      x = fma(-CHEM_LDLU(lu + 97), b[35], x);
      x = fma(-CHEM_LDLU(lu + 98), b[36], x);
      b[112] = x;
    }
    {
      double x = b[113];
      x = fma(-CHEM_LDLU(lu + 99), b[12], x);
      x = fma(-CHEM_LDLU(lu + 100), b[34], x);
      x = fma(-CHEM_LDLU(lu + 101), b[35], x);
      x = fma(-CHEM_LDLU(lu + 102), b[36], x);
      x = fma(-CHEM_LDLU(lu + 103), b[104], x);
      b[113] = x;
    }
    {
      double x = b[114];
      x = fma(-CHEM_LDLU(lu + 104), b[30], x);
      x = fma(-CHEM_LDLU(lu + 105), b[62], x);
      x = fma(-CHEM_LDLU(lu + 106), b[83], x);
      x = fma(-CHEM_LDLU(lu + 107), b[98], x);
      x = fma(-CHEM_LDLU(lu + 108), b[107], x);
      x = fma(-CHEM_LDLU(lu + 109), b[111], x);
      b[114] = x;
    }
    {
      double x = b[115];
      x = fma(-CHEM_LDLU(lu + 110), b[47], x);
      x = fma(-CHEM_LDLU(lu + 111), b[72], x);
      x = fma(-CHEM_LDLU(lu + 112), b[86], x);
      x = fma(-CHEM_LDLU(lu + 113), b[87], x);
      x = fma(-CHEM_LDLU(lu + 114), b[88], x);
      x = fma(-CHEM_LDLU(lu + 115), b[91], x);
      x = fma(-CHEM_LDLU(lu + 116), b[99], x);
      x = fma(-CHEM_LDLU(lu + 117), b[100], x);
      b[115] = x;
    }
    {
      double x = b[116];
      x = fma(-CHEM_LDLU(lu + 118), b[47], x);
      x = fma(-CHEM_LDLU(lu + 119), b[72], x);
      x = fma(-CHEM_LDLU(lu + 120), b[86], x);
      x = fma(-CHEM_LDLU(lu + 121), b[87], x);
      x = fma(-CHEM_LDLU(lu + 122), b[88], x);
      x = fma(-CHEM_LDLU(lu + 123), b[91], x);
      x = fma(-CHEM_LDLU(lu + 124), b[99], x);
      x = fma(-CHEM_LDLU(lu + 125), b[100], x);
      x = fma(-CHEM_LDLU(lu + 126), b[115], x);
      b[116] = x;
    }
    {
      double x = b[117];
      x = fma(-CHEM_LDLU(lu + 127), b[56], x);
      x = fma(-CHEM_LDLU(lu + 128), b[113], x);
      b[117] = x;
    }
    {
      double x = b[118];
      x = fma(-CHEM_LDLU(lu + 129), b[11], x);
      x = fma(-CHEM_LDLU(lu + 130), b[51], x);
      x = fma(-CHEM_LDLU(lu + 131), b[54], x);
      x = fma(-CHEM_LDLU(lu + 132), b[83], x);
      x = fma(-CHEM_LDLU(lu + 133), b[103], x);
      x = fma(-CHEM_LDLU(lu + 134), b[107], x);
      x = fma(-CHEM_LDLU(lu + 135), b[111], x);
      b[118] = x;
    }
    {
      double x = b[119];
      x = fma(-CHEM_LDLU(lu + 136), b[35], x);
      x = fma(-CHEM_LDLU(lu + 137), b[36], x);
      x = fma(-CHEM_LDLU(lu + 138), b[109], x);
      x = fma(-CHEM_LDLU(lu + 139), b[112], x);
      b[119] = x;
    }
    {
      double x = b[120];
      x = fma(-CHEM_LDLU(lu + 140), b[27], x);
      x = fma(-CHEM_LDLU(lu + 141), b[51], x);
      x = fma(-CHEM_LDLU(lu + 142), b[83], x);
      x = fma(-CHEM_LDLU(lu + 143), b[103], x);
      x = fma(-CHEM_LDLU(lu + 144), b[107], x);
      b[120] = x;
    }
    {
      double x = b[121];
      x = fma(-CHEM_LDLU(lu + 145), b[32], x);
      x = fma(-CHEM_LDLU(lu + 146), b[79], x);
      x = fma(-CHEM_LDLU(lu + 147), b[107], x);
      b[121] = x;
    }
    {
      double x = b[122];
      x = fma(-CHEM_LDLU(lu + 148), b[98], x);
      x = fma(-CHEM_LDLU(lu + 149), b[103], x);
      x = fma(-CHEM_LDLU(lu + 150), b[107], x);
      x = fma(-CHEM_LDLU(lu + 151), b[111], x);
      x = fma(-CHEM_LDLU(lu + 152), b[117], x);
      x = fma(-CHEM_LDLU(lu + 153), b[121], x);
      b[122] = x;
    }
    {
      double x = b[123];
      x = fma(-CHEM_LDLU(lu + 154), b[12], x);
      x = fma(-CHEM_LDLU(lu + 155), b[34], x);
      x = fma(-CHEM_LDLU(lu + 156), b[68], x);
      x = fma(-CHEM_LDLU(lu + 157), b[97], x);
      x = fma(-CHEM_LDLU(lu + 158), b[104], x);
      x = fma(-CHEM_LDLU(lu + 159), b[109], x);
      x = fma(-CHEM_LDLU(lu + 160), b[112], x);
      x = fma(-CHEM_LDLU(lu + 161), b[113], x);
      x = fma(-CHEM_LDLU(lu + 162), b[119], x);
      b[123] = x;
    }
    {
      double x = b[124];
      x = fma(-CHEM_LDLU(lu + 163), b[26], x);
      x = fma(-CHEM_LDLU(lu + 164), b[27], x);
      x = fma(-CHEM_LDLU(lu + 165), b[28], x);
      x = fma(-CHEM_LDLU(lu + 166), b[34], x);
      x = fma(-CHEM_LDLU(lu + 167), b[35], x);
      x = fma(-CHEM_LDLU(lu + 168), b[36], x);
      x = fma(-CHEM_LDLU(lu + 169), b[63], x);
      x = fma(-CHEM_LDLU(lu + 170), b[85], x);
      x = fma(-CHEM_LDLU(lu + 171), b[98], x);
      x = fma(-CHEM_LDLU(lu + 172), b[107], x);
      x = fma(-CHEM_LDLU(lu + 173), b[120], x);
      x = fma(-CHEM_LDLU(lu + 174), b[121], x);
      b[124] = x;
    }
    {
      double x = b[125];
      x = fma(-CHEM_LDLU(lu + 175), b[98], x);
      x = fma(-CHEM_LDLU(lu + 176), b[103], x);
      x = fma(-CHEM_LDLU(lu + 177), b[107], x);
      x = fma(-CHEM_LDLU(lu + 178), b[109], x);
      x = fma(-CHEM_LDLU(lu + 179), b[111], x);
      x = fma(-CHEM_LDLU(lu + 180), b[112], x);
      x = fma(-CHEM_LDLU(lu + 181), b[113], x);
      x = fma(-CHEM_LDLU(lu + 182), b[119], x);
      x = fma(-CHEM_LDLU(lu + 183), b[121], x);
      x = fma(-CHEM_LDLU(lu + 184), b[123], x);
      b[125] = x;
    }
    {
      double x = b[126];
      x = fma(-CHEM_LDLU(lu + 185), b[51], x);
      x = fma(-CHEM_LDLU(lu + 186), b[56], x);
      x = fma(-CHEM_LDLU(lu + 187), b[64], x);
      x = fma(-CHEM_LDLU(lu + 188), b[66], x);
      x = fma(-CHEM_LDLU(lu + 189), b[68], x);
      x = fma(-CHEM_LDLU(lu + 190), b[79], x);
      x = fma(-CHEM_LDLU(lu + 191), b[97], x);
      x = fma(-CHEM_LDLU(lu + 192), b[104], x);
      x = fma(-CHEM_LDLU(lu + 193), b[107], x);
      x = fma(-CHEM_LDLU(lu + 194), b[109], x);
      x = fma(-CHEM_LDLU(lu + 195), b[112], x);
      x = fma(-CHEM_LDLU(lu + 196), b[113], x);
      x = fma(-CHEM_LDLU(lu + 197), b[114], x);
      x = fma(-CHEM_LDLU(lu + 198), b[117], x);
      x = fma(-CHEM_LDLU(lu + 199), b[119], x);
      x = fma(-CHEM_LDLU(lu + 200), b[121], x);
      x = fma(-CHEM_LDLU(lu + 201), b[123], x);
      b[126] = x;
    }
    {
      double x = b[127];
      x = fma(-CHEM_LDLU(lu + 202), b[29], x);
      x = fma(-CHEM_LDLU(lu + 203), b[30], x);
      x = fma(-CHEM_LDLU(lu + 204), b[51], x);
      x = fma(-CHEM_LDLU(lu + 205), b[52], x);
      x = fma(-CHEM_LDLU(lu + 206), b[62], x);
      x = fma(-CHEM_LDLU(lu + 207), b[64], x);
      x = fma(-CHEM_LDLU(lu + 208), b[66], x);
      x = fma(-CHEM_LDLU(lu + 209), b[79], x);
      x = fma(-CHEM_LDLU(lu + 210), b[98], x);
      x = fma(-CHEM_LDLU(lu + 211), b[107], x);
      x = fma(-CHEM_LDLU(lu + 212), b[111], x);
      x = fma(-CHEM_LDLU(lu + 213), b[117], x);
      x = fma(-CHEM_LDLU(lu + 214), b[121], x);
      x = fma(-CHEM_LDLU(lu + 215), b[123], x);
      b[127] = x;
    }
    {
      double x = b[128];
      x = fma(-CHEM_LDLU(lu + 216), b[10], x);
      x = fma(-CHEM_LDLU(lu + 217), b[30], x);
      x = fma(-CHEM_LDLU(lu + 218), b[61], x);
      x = fma(-CHEM_LDLU(lu + 219), b[62], x);
      x = fma(-CHEM_LDLU(lu + 220), b[64], x);
      x = fma(-CHEM_LDLU(lu + 221), b[66], x);
      x = fma(-CHEM_LDLU(lu + 222), b[79], x);
      x = fma(-CHEM_LDLU(lu + 223), b[117], x);
      x = fma(-CHEM_LDLU(lu + 224), b[121], x);
      x = fma(-CHEM_LDLU(lu + 225), b[123], x);
      x = fma(-CHEM_LDLU(lu + 226), b[127], x);
      b[128] = x;
    }
    {
      double x = b[129];
      x = fma(-CHEM_LDLU(lu + 227), b[10], x);
      x = fma(-CHEM_LDLU(lu + 228), b[26], x);
      x = fma(-CHEM_LDLU(lu + 229), b[27], x);
      x = fma(-CHEM_LDLU(lu + 230), b[30], x);
      x = fma(-CHEM_LDLU(lu + 231), b[61], x);
      x = fma(-CHEM_LDLU(lu + 232), b[62], x);
      x = fma(-CHEM_LDLU(lu + 233), b[98], x);
      x = fma(-CHEM_LDLU(lu + 234), b[107], x);
      x = fma(-CHEM_LDLU(lu + 235), b[111], x);
      x = fma(-CHEM_LDLU(lu + 236), b[119], x);
      x = fma(-CHEM_LDLU(lu + 237), b[121], x);
      x = fma(-CHEM_LDLU(lu + 238), b[123], x);
      x = fma(-CHEM_LDLU(lu + 239), b[127], x);
      x = fma(-CHEM_LDLU(lu + 240), b[128], x);
      b[129] = x;
    }
    {
      double x = b[130];
      x = fma(-CHEM_LDLU(lu + 241), b[21], x);
      x = fma(-CHEM_LDLU(lu + 242), b[64], x);
      x = fma(-CHEM_LDLU(lu + 243), b[66], x);
      x = fma(-CHEM_LDLU(lu + 244), b[73], x);
      x = fma(-CHEM_LDLU(lu + 245), b[74], x);
      x = fma(-CHEM_LDLU(lu + 246), b[79], x);
      x = fma(-CHEM_LDLU(lu + 247), b[83], x);
      x = fma(-CHEM_LDLU(lu + 248), b[98], x);
      x = fma(-CHEM_LDLU(lu + 249), b[107], x);
      x = fma(-CHEM_LDLU(lu + 250), b[108], x);
      x = fma(-CHEM_LDLU(lu + 251), b[110], x);
      x = fma(-CHEM_LDLU(lu + 252), b[111], x);
      x = fma(-CHEM_LDLU(lu + 253), b[121], x);
      x = fma(-CHEM_LDLU(lu + 254), b[127], x);
      x = fma(-CHEM_LDLU(lu + 255), b[129], x);
      b[130] = x;
    }
    {
      double x = b[131];
      x = fma(-CHEM_LDLU(lu + 256), b[32], x);
      x = fma(-CHEM_LDLU(lu + 257), b[38], x);
      x = fma(-CHEM_LDLU(lu + 258), b[39], x);
      x = fma(-CHEM_LDLU(lu + 259), b[40], x);
      x = fma(-CHEM_LDLU(lu + 260), b[55], x);
      x = fma(-CHEM_LDLU(lu + 261), b[60], x);
      x = fma(-CHEM_LDLU(lu + 262), b[63], x);
      x = fma(-CHEM_LDLU(lu + 263), b[68], x);
      x = fma(-CHEM_LDLU(lu + 264), b[104], x);
      x = fma(-CHEM_LDLU(lu + 265), b[107], x);
      x = fma(-CHEM_LDLU(lu + 266), b[110], x);
      x = fma(-CHEM_LDLU(lu + 267), b[113], x);
      x = fma(-CHEM_LDLU(lu + 268), b[120], x);
      x = fma(-CHEM_LDLU(lu + 269), b[121], x);
      x = fma(-CHEM_LDLU(lu + 270), b[123], x);
      x = fma(-CHEM_LDLU(lu + 271), b[125], x);
      x = fma(-CHEM_LDLU(lu + 272), b[126], x);
      x = fma(-CHEM_LDLU(lu + 273), b[127], x);
      x = fma(-CHEM_LDLU(lu + 274), b[129], x);
      x = fma(-CHEM_LDLU(lu + 275), b[130], x);
      b[131] = x;
    }
    {
      double x = b[132];
      x = fma(-CHEM_LDLU(lu + 276), b[10], x);
      x = fma(-CHEM_LDLU(lu + 277), b[29], x);
      x = fma(-CHEM_LDLU(lu + 278), b[30], x);
      x = fma(-CHEM_LDLU(lu + 279), b[51], x);
      x = fma(-CHEM_LDLU(lu + 280), b[62], x);
      x = fma(-CHEM_LDLU(lu + 281), b[64], x);
      x = fma(-CHEM_LDLU(lu + 282), b[66], x);
      x = fma(-CHEM_LDLU(lu + 283), b[79], x);
      x = fma(-CHEM_LDLU(lu + 284), b[98], x);
      x = fma(-CHEM_LDLU(lu + 285), b[103], x);
      x = fma(-CHEM_LDLU(lu + 286), b[107], x);
      x = fma(-CHEM_LDLU(lu + 287), b[111], x);
      x = fma(-CHEM_LDLU(lu + 288), b[121], x);
      x = fma(-CHEM_LDLU(lu + 289), b[130], x);
      b[132] = x;
    }
    {
      double x = b[133];
      x = fma(-CHEM_LDLU(lu + 290), b[11], x);
      x = fma(-CHEM_LDLU(lu + 291), b[56], x);
      x = fma(-CHEM_LDLU(lu + 292), b[97], x);
      x = fma(-CHEM_LDLU(lu + 293), b[98], x);
      x = fma(-CHEM_LDLU(lu + 294), b[103], x);
      x = fma(-CHEM_LDLU(lu + 295), b[107], x);
      x = fma(-CHEM_LDLU(lu + 296), b[109], x);
      x = fma(-CHEM_LDLU(lu + 297), b[111], x);
      x = fma(-CHEM_LDLU(lu + 298), b[112], x);
      x = fma(-CHEM_LDLU(lu + 299), b[113], x);
      x = fma(-CHEM_LDLU(lu + 300), b[117], x);
      x = fma(-CHEM_LDLU(lu + 301), b[119], x);
      x = fma(-CHEM_LDLU(lu + 302), b[120], x);
      x = fma(-CHEM_LDLU(lu + 303), b[121], x);
      x = fma(-CHEM_LDLU(lu + 304), b[123], x);
      x = fma(-CHEM_LDLU(lu + 305), b[130], x);
      x = fma(-CHEM_LDLU(lu + 306), b[132], x);
      b[133] = x;
    }
    {
      double x = b[134];
      x = fma(-CHEM_LDLU(lu + 307), b[26], x);
      x = fma(-CHEM_LDLU(lu + 308), b[28], x);
      x = fma(-CHEM_LDLU(lu + 309), b[29], x);
      x = fma(-CHEM_LDLU(lu + 310), b[30], x);
      x = fma(-CHEM_LDLU(lu + 311), b[62], x);
      x = fma(-CHEM_LDLU(lu + 312), b[64], x);
      x = fma(-CHEM_LDLU(lu + 313), b[66], x);
      x = fma(-CHEM_LDLU(lu + 314), b[79], x);
      x = fma(-CHEM_LDLU(lu + 315), b[90], x);
      x = fma(-CHEM_LDLU(lu + 316), b[98], x);
      x = fma(-CHEM_LDLU(lu + 317), b[107], x);
      x = fma(-CHEM_LDLU(lu + 318), b[111], x);
      x = fma(-CHEM_LDLU(lu + 319), b[113], x);
      x = fma(-CHEM_LDLU(lu + 320), b[119], x);
      x = fma(-CHEM_LDLU(lu + 321), b[121], x);
      x = fma(-CHEM_LDLU(lu + 322), b[130], x);
      x = fma(-CHEM_LDLU(lu + 323), b[132], x);
      b[134] = x;
    }
    {
      double x = b[135];
      x = fma(-CHEM_LDLU(lu + 324), b[58], x);
      x = fma(-CHEM_LDLU(lu + 325), b[64], x);
      x = fma(-CHEM_LDLU(lu + 326), b[66], x);
      x = fma(-CHEM_LDLU(lu + 327), b[75], x);
      x = fma(-CHEM_LDLU(lu + 328), b[76], x);
      x = fma(-CHEM_LDLU(lu + 329), b[79], x);
      x = fma(-CHEM_LDLU(lu + 330), b[83], x);
      x = fma(-CHEM_LDLU(lu + 331), b[93], x);
      x = fma(-CHEM_LDLU(lu + 332), b[94], x);
      x = fma(-CHEM_LDLU(lu + 333), b[98], x);
      x = fma(-CHEM_LDLU(lu + 334), b[107], x);
      x = fma(-CHEM_LDLU(lu + 335), b[108], x);
      x = fma(-CHEM_LDLU(lu + 336), b[110], x);
      x = fma(-CHEM_LDLU(lu + 337), b[111], x);
      x = fma(-CHEM_LDLU(lu + 338), b[117], x);
      x = fma(-CHEM_LDLU(lu + 339), b[119], x);
      x = fma(-CHEM_LDLU(lu + 340), b[121], x);
      x = fma(-CHEM_LDLU(lu + 341), b[123], x);
      x = fma(-CHEM_LDLU(lu + 342), b[128], x);
      x = fma(-CHEM_LDLU(lu + 343), b[130], x);
      x = fma(-CHEM_LDLU(lu + 344), b[132], x);
      b[135] = x;
    }
    {
      double x = b[136];
      x = fma(-CHEM_LDLU(lu + 345), b[51], x);
      x = fma(-CHEM_LDLU(lu + 346), b[62], x);
      x = fma(-CHEM_LDLU(lu + 347), b[64], x);
      x = fma(-CHEM_LDLU(lu + 348), b[66], x);
      x = fma(-CHEM_LDLU(lu + 349), b[79], x);
      x = fma(-CHEM_LDLU(lu + 350), b[83], x);
      x = fma(-CHEM_LDLU(lu + 351), b[98], x);
      x = fma(-CHEM_LDLU(lu + 352), b[106], x);
      x = fma(-CHEM_LDLU(lu + 353), b[107], x);
      x = fma(-CHEM_LDLU(lu + 354), b[111], x);
      x = fma(-CHEM_LDLU(lu + 355), b[113], x);
      x = fma(-CHEM_LDLU(lu + 356), b[117], x);
      x = fma(-CHEM_LDLU(lu + 357), b[119], x);
      x = fma(-CHEM_LDLU(lu + 358), b[121], x);
      x = fma(-CHEM_LDLU(lu + 359), b[123], x);
      x = fma(-CHEM_LDLU(lu + 360), b[125], x);
      x = fma(-CHEM_LDLU(lu + 361), b[130], x);
      x = fma(-CHEM_LDLU(lu + 362), b[132], x);
      x = fma(-CHEM_LDLU(lu + 363), b[133], x);
      x = fma(-CHEM_LDLU(lu + 364), b[135], x);
      b[136] = x;
    }
    {
      double x = b[137];
      x = fma(-CHEM_LDLU(lu + 365), b[54], x);
      x = fma(-CHEM_LDLU(lu + 366), b[67], x);
      x = fma(-CHEM_LDLU(lu + 367), b[77], x);
      x = fma(-CHEM_LDLU(lu + 368), b[78], x);
      x = fma(-CHEM_LDLU(lu + 369), b[80], x);
      x = fma(-CHEM_LDLU(lu + 370), b[89], x);
      x = fma(-CHEM_LDLU(lu + 371), b[92], x);
      x = fma(-CHEM_LDLU(lu + 372), b[97], x);
      x = fma(-CHEM_LDLU(lu + 373), b[103], x);
      x = fma(-CHEM_LDLU(lu + 374), b[104], x);
      x = fma(-CHEM_LDLU(lu + 375), b[107], x);
      x = fma(-CHEM_LDLU(lu + 376), b[109], x);
      x = fma(-CHEM_LDLU(lu + 377), b[110], x);
      x = fma(-CHEM_LDLU(lu + 378), b[112], x);
      x = fma(-CHEM_LDLU(lu + 379), b[113], x);
      x = fma(-CHEM_LDLU(lu + 380), b[117], x);
      x = fma(-CHEM_LDLU(lu + 381), b[121], x);
      x = fma(-CHEM_LDLU(lu + 382), b[123], x);
      x = fma(-CHEM_LDLU(lu + 383), b[128], x);
      x = fma(-CHEM_LDLU(lu + 384), b[130], x);
      x = fma(-CHEM_LDLU(lu + 385), b[132], x);
      x = fma(-CHEM_LDLU(lu + 386), b[134], x);
      x = fma(-CHEM_LDLU(lu + 387), b[135], x);
      x = fma(-CHEM_LDLU(lu + 388), b[136], x);
      b[137] = x;
    }
    {
      double x = b[138];
      x = fma(-CHEM_LDLU(lu + 389), b[10], x);
      x = fma(-CHEM_LDLU(lu + 390), b[13], x);
      x = fma(-CHEM_LDLU(lu + 391), b[30], x);
      x = fma(-CHEM_LDLU(lu + 392), b[42], x);
      x = fma(-CHEM_LDLU(lu + 393), b[62], x);
      x = fma(-CHEM_LDLU(lu + 394), b[63], x);
      x = fma(-CHEM_LDLU(lu + 395), b[71], x);
      x = fma(-CHEM_LDLU(lu + 396), b[97], x);
      x = fma(-CHEM_LDLU(lu + 397), b[103], x);
      x = fma(-CHEM_LDLU(lu + 398), b[106], x);
      x = fma(-CHEM_LDLU(lu + 399), b[107], x);
      x = fma(-CHEM_LDLU(lu + 400), b[109], x);
      x = fma(-CHEM_LDLU(lu + 401), b[110], x);
      x = fma(-CHEM_LDLU(lu + 402), b[112], x);
      x = fma(-CHEM_LDLU(lu + 403), b[117], x);
      x = fma(-CHEM_LDLU(lu + 404), b[121], x);
      x = fma(-CHEM_LDLU(lu + 405), b[122], x);
      x = fma(-CHEM_LDLU(lu + 406), b[123], x);
      x = fma(-CHEM_LDLU(lu + 407), b[128], x);
      x = fma(-CHEM_LDLU(lu + 408), b[129], x);
      x = fma(-CHEM_LDLU(lu + 409), b[130], x);
      x = fma(-CHEM_LDLU(lu + 410), b[132], x);
      x = fma(-CHEM_LDLU(lu + 411), b[134], x);
      x = fma(-CHEM_LDLU(lu + 412), b[135], x);
      x = fma(-CHEM_LDLU(lu + 413), b[136], x);
      x = fma(-CHEM_LDLU(lu + 414), b[137], x);
      b[138] = x;
    }
    {
      double x = b[139];
      x = fma(-CHEM_LDLU(lu + 415), b[10], x);
      x = fma(-CHEM_LDLU(lu + 416), b[30], x);
      x = fma(-CHEM_LDLU(lu + 417), b[42], x);
      x = fma(-CHEM_LDLU(lu + 418), b[62], x);
      x = fma(-CHEM_LDLU(lu + 419), b[84], x);
      x = fma(-CHEM_LDLU(lu + 420), b[97], x);
      x = fma(-CHEM_LDLU(lu + 421), b[103], x);
      x = fma(-CHEM_LDLU(lu + 422), b[106], x);
      x = fma(-CHEM_LDLU(lu + 423), b[107], x);
      x = fma(-CHEM_LDLU(lu + 424), b[109], x);
      x = fma(-CHEM_LDLU(lu + 425), b[112], x);
      x = fma(-CHEM_LDLU(lu + 426), b[117], x);
      x = fma(-CHEM_LDLU(lu + 427), b[119], x);
      x = fma(-CHEM_LDLU(lu + 428), b[120], x);
      x = fma(-CHEM_LDLU(lu + 429), b[121], x);
      x = fma(-CHEM_LDLU(lu + 430), b[123], x);
      x = fma(-CHEM_LDLU(lu + 431), b[125], x);
      x = fma(-CHEM_LDLU(lu + 432), b[128], x);
      x = fma(-CHEM_LDLU(lu + 433), b[129], x);
      x = fma(-CHEM_LDLU(lu + 434), b[130], x);
      x = fma(-CHEM_LDLU(lu + 435), b[132], x);
      x = fma(-CHEM_LDLU(lu + 436), b[134], x);
      x = fma(-CHEM_LDLU(lu + 437), b[135], x);
      x = fma(-CHEM_LDLU(lu + 438), b[136], x);
      x = fma(-CHEM_LDLU(lu + 439), b[137], x);
      x = fma(-CHEM_LDLU(lu + 440), b[138], x);
      b[139] = x;
    }
    {
      double x = b[140];
      x = fma(-CHEM_LDLU(lu + 441), b[11], x);
      x = fma(-CHEM_LDLU(lu + 442), b[56], x);
      x = fma(-CHEM_LDLU(lu + 443), b[64], x);
      x = fma(-CHEM_LDLU(lu + 444), b[66], x);
      x = fma(-CHEM_LDLU(lu + 445), b[79], x);
      x = fma(-CHEM_LDLU(lu + 446), b[83], x);
      x = fma(-CHEM_LDLU(lu + 447), b[98], x);
      x = fma(-CHEM_LDLU(lu + 448), b[101], x);
      x = fma(-CHEM_LDLU(lu + 449), b[103], x);
      x = fma(-CHEM_LDLU(lu + 450), b[106], x);
      x = fma(-CHEM_LDLU(lu + 451), b[107], x);
      x = fma(-CHEM_LDLU(lu + 452), b[111], x);
      x = fma(-CHEM_LDLU(lu + 453), b[117], x);
      x = fma(-CHEM_LDLU(lu + 454), b[119], x);
      x = fma(-CHEM_LDLU(lu + 455), b[120], x);
      x = fma(-CHEM_LDLU(lu + 456), b[121], x);
      x = fma(-CHEM_LDLU(lu + 457), b[123], x);
      x = fma(-CHEM_LDLU(lu + 458), b[125], x);
      x = fma(-CHEM_LDLU(lu + 459), b[127], x);
      x = fma(-CHEM_LDLU(lu + 460), b[129], x);
      x = fma(-CHEM_LDLU(lu + 461), b[130], x);
      x = fma(-CHEM_LDLU(lu + 462), b[132], x);
      x = fma(-CHEM_LDLU(lu + 463), b[133], x);
      x = fma(-CHEM_LDLU(lu + 464), b[135], x);
      x = fma(-CHEM_LDLU(lu + 465), b[137], x);
      x = fma(-CHEM_LDLU(lu + 466), b[138], x);
      x = fma(-CHEM_LDLU(lu + 467), b[139], x);
      b[140] = x;
    }
    {
      double x = b[141];
      x = fma(-CHEM_LDLU(lu + 468), b[27], x);
      x = fma(-CHEM_LDLU(lu + 469), b[51], x);
      x = fma(-CHEM_LDLU(lu + 470), b[54], x);
      x = fma(-CHEM_LDLU(lu + 471), b[55], x);
      x = fma(-CHEM_LDLU(lu + 472), b[63], x);
      x = fma(-CHEM_LDLU(lu + 473), b[64], x);
      x = fma(-CHEM_LDLU(lu + 474), b[66], x);
      x = fma(-CHEM_LDLU(lu + 475), b[68], x);
      x = fma(-CHEM_LDLU(lu + 476), b[71], x);
      x = fma(-CHEM_LDLU(lu + 477), b[79], x);
      x = fma(-CHEM_LDLU(lu + 478), b[83], x);
      x = fma(-CHEM_LDLU(lu + 479), b[85], x);
      x = fma(-CHEM_LDLU(lu + 480), b[98], x);
      x = fma(-CHEM_LDLU(lu + 481), b[103], x);
      x = fma(-CHEM_LDLU(lu + 482), b[104], x);
      x = fma(-CHEM_LDLU(lu + 483), b[106], x);
      x = fma(-CHEM_LDLU(lu + 484), b[107], x);
      x = fma(-CHEM_LDLU(lu + 485), b[110], x);
      x = fma(-CHEM_LDLU(lu + 486), b[111], x);
      x = fma(-CHEM_LDLU(lu + 487), b[113], x);
      x = fma(-CHEM_LDLU(lu + 488), b[120], x);
      x = fma(-CHEM_LDLU(lu + 489), b[121], x);
      x = fma(-CHEM_LDLU(lu + 490), b[123], x);
      x = fma(-CHEM_LDLU(lu + 491), b[130], x);
      x = fma(-CHEM_LDLU(lu + 492), b[132], x);
      x = fma(-CHEM_LDLU(lu + 493), b[135], x);
      x = fma(-CHEM_LDLU(lu + 494), b[137], x);
      x = fma(-CHEM_LDLU(lu + 495), b[138], x);
      x = fma(-CHEM_LDLU(lu + 496), b[139], x);
      b[141] = x;
    }
    {
      double x = b[142];
      x = fma(-CHEM_LDLU(lu + 497), b[26], x);
      x = fma(-CHEM_LDLU(lu + 498), b[27], x);
      x = fma(-CHEM_LDLU(lu + 499), b[28], x);
      x = fma(-CHEM_LDLU(lu + 500), b[34], x);
      x = fma(-CHEM_LDLU(lu + 501), b[35], x);
      x = fma(-CHEM_LDLU(lu + 502), b[36], x);
      x = fma(-CHEM_LDLU(lu + 503), b[37], x);
      x = fma(-CHEM_LDLU(lu + 504), b[38], x);
      x = fma(-CHEM_LDLU(lu + 505), b[48], x);
      x = fma(-CHEM_LDLU(lu + 506), b[57], x);
      x = fma(-CHEM_LDLU(lu + 507), b[63], x);
      x = fma(-CHEM_LDLU(lu + 508), b[73], x);
      x = fma(-CHEM_LDLU(lu + 509), b[74], x);
      x = fma(-CHEM_LDLU(lu + 510), b[75], x);
      x = fma(-CHEM_LDLU(lu + 511), b[76], x);
      x = fma(-CHEM_LDLU(lu + 512), b[79], x);
      x = fma(-CHEM_LDLU(lu + 513), b[81], x);
      x = fma(-CHEM_LDLU(lu + 514), b[83], x);
      x = fma(-CHEM_LDLU(lu + 515), b[85], x);
      x = fma(-CHEM_LDLU(lu + 516), b[93], x);
      x = fma(-CHEM_LDLU(lu + 517), b[94], x);
      x = fma(-CHEM_LDLU(lu + 518), b[98], x);
      x = fma(-CHEM_LDLU(lu + 519), b[101], x);
      x = fma(-CHEM_LDLU(lu + 520), b[105], x);
      x = fma(-CHEM_LDLU(lu + 521), b[107], x);
      x = fma(-CHEM_LDLU(lu + 522), b[108], x);
      x = fma(-CHEM_LDLU(lu + 523), b[110], x);
      x = fma(-CHEM_LDLU(lu + 524), b[111], x);
      x = fma(-CHEM_LDLU(lu + 525), b[120], x);
      x = fma(-CHEM_LDLU(lu + 526), b[121], x);
      x = fma(-CHEM_LDLU(lu + 527), b[124], x);
      x = fma(-CHEM_LDLU(lu + 528), b[127], x);
      x = fma(-CHEM_LDLU(lu + 529), b[129], x);
      x = fma(-CHEM_LDLU(lu + 530), b[130], x);
      x = fma(-CHEM_LDLU(lu + 531), b[132], x);
      x = fma(-CHEM_LDLU(lu + 532), b[135], x);
      x = fma(-CHEM_LDLU(lu + 533), b[137], x);
      x = fma(-CHEM_LDLU(lu + 534), b[138], x);
      x = fma(-CHEM_LDLU(lu + 535), b[139], x);
      x = fma(-CHEM_LDLU(lu + 536), b[141], x);
      b[142] = x;
    }
    {
      double x = b[143];
      x = fma(-CHEM_LDLU(lu + 537), b[10], x);
      x = fma(-CHEM_LDLU(lu + 538), b[26], x);
      x = fma(-CHEM_LDLU(lu + 539), b[27], x);
      x = fma(-CHEM_LDLU(lu + 540), b[28], x);
      x = fma(-CHEM_LDLU(lu + 541), b[29], x);
      x = fma(-CHEM_LDLU(lu + 542), b[30], x);
      x = fma(-CHEM_LDLU(lu + 543), b[34], x);
      x = fma(-CHEM_LDLU(lu + 544), b[35], x);
      x = fma(-CHEM_LDLU(lu + 545), b[36], x);
      x = fma(-CHEM_LDLU(lu + 546), b[51], x);
      x = fma(-CHEM_LDLU(lu + 547), b[61], x);
      x = fma(-CHEM_LDLU(lu + 548), b[62], x);
      x = fma(-CHEM_LDLU(lu + 549), b[64], x);
      x = fma(-CHEM_LDLU(lu + 550), b[66], x);
      x = fma(-CHEM_LDLU(lu + 551), b[79], x);
      x = fma(-CHEM_LDLU(lu + 552), b[83], x);
      x = fma(-CHEM_LDLU(lu + 553), b[90], x);
      x = fma(-CHEM_LDLU(lu + 554), b[98], x);
      x = fma(-CHEM_LDLU(lu + 555), b[107], x);
      x = fma(-CHEM_LDLU(lu + 556), b[111], x);
      x = fma(-CHEM_LDLU(lu + 557), b[113], x);
      x = fma(-CHEM_LDLU(lu + 558), b[117], x);
      x = fma(-CHEM_LDLU(lu + 559), b[119], x);
      x = fma(-CHEM_LDLU(lu + 560), b[120], x);
      x = fma(-CHEM_LDLU(lu + 561), b[121], x);
      x = fma(-CHEM_LDLU(lu + 562), b[123], x);
      x = fma(-CHEM_LDLU(lu + 563), b[127], x);
      x = fma(-CHEM_LDLU(lu + 564), b[128], x);
      x = fma(-CHEM_LDLU(lu + 565), b[130], x);
      x = fma(-CHEM_LDLU(lu + 566), b[132], x);
      x = fma(-CHEM_LDLU(lu + 567), b[134], x);
      x = fma(-CHEM_LDLU(lu + 568), b[135], x);
      x = fma(-CHEM_LDLU(lu + 569), b[136], x);
      x = fma(-CHEM_LDLU(lu + 570), b[137], x);
      x = fma(-CHEM_LDLU(lu + 571), b[138], x);
      x = fma(-CHEM_LDLU(lu + 572), b[139], x);
      x = fma(-CHEM_LDLU(lu + 573), b[141], x);
      x = fma(-CHEM_LDLU(lu + 574), b[142], x);
      b[143] = x;
    }
    {
      double x = b[144];
      x = fma(-CHEM_LDLU(lu + 575), b[30], x);
      x = fma(-CHEM_LDLU(lu + 576), b[38], x);
      x = fma(-CHEM_LDLU(lu + 577), b[40], x);
      x = fma(-CHEM_LDLU(lu + 578), b[42], x);
      x = fma(-CHEM_LDLU(lu + 579), b[51], x);
      x = fma(-CHEM_LDLU(lu + 580), b[53], x);
      x = fma(-CHEM_LDLU(lu + 581), b[54], x);
      x = fma(-CHEM_LDLU(lu + 582), b[56], x);
      x = fma(-CHEM_LDLU(lu + 583), b[61], x);
      x = fma(-CHEM_LDLU(lu + 584), b[62], x);
      x = fma(-CHEM_LDLU(lu + 585), b[64], x);
      x = fma(-CHEM_LDLU(lu + 586), b[66], x);
      x = fma(-CHEM_LDLU(lu + 587), b[77], x);
      x = fma(-CHEM_LDLU(lu + 588), b[79], x);
      x = fma(-CHEM_LDLU(lu + 589), b[81], x);
      x = fma(-CHEM_LDLU(lu + 590), b[83], x);
      x = fma(-CHEM_LDLU(lu + 591), b[97], x);
      x = fma(-CHEM_LDLU(lu + 592), b[98], x);
      x = fma(-CHEM_LDLU(lu + 593), b[103], x);
      x = fma(-CHEM_LDLU(lu + 594), b[104], x);
      x = fma(-CHEM_LDLU(lu + 595), b[107], x);
      x = fma(-CHEM_LDLU(lu + 596), b[109], x);
      x = fma(-CHEM_LDLU(lu + 597), b[110], x);
      x = fma(-CHEM_LDLU(lu + 598), b[111], x);
      x = fma(-CHEM_LDLU(lu + 599), b[112], x);
      x = fma(-CHEM_LDLU(lu + 600), b[113], x);
      x = fma(-CHEM_LDLU(lu + 601), b[114], x);
      x = fma(-CHEM_LDLU(lu + 602), b[117], x);
      x = fma(-CHEM_LDLU(lu + 603), b[119], x);
      x = fma(-CHEM_LDLU(lu + 604), b[121], x);
      x = fma(-CHEM_LDLU(lu + 605), b[123], x);
      x = fma(-CHEM_LDLU(lu + 606), b[128], x);
      x = fma(-CHEM_LDLU(lu + 607), b[130], x);
      x = fma(-CHEM_LDLU(lu + 608), b[131], x);
      x = fma(-CHEM_LDLU(lu + 609), b[132], x);
      x = fma(-CHEM_LDLU(lu + 610), b[133], x);
      x = fma(-CHEM_LDLU(lu + 611), b[134], x);
      x = fma(-CHEM_LDLU(lu + 612), b[135], x);
      x = fma(-CHEM_LDLU(lu + 613), b[136], x);
      x = fma(-CHEM_LDLU(lu + 614), b[137], x);
      x = fma(-CHEM_LDLU(lu + 615), b[138], x);
      x = fma(-CHEM_LDLU(lu + 616), b[139], x);
      x = fma(-CHEM_LDLU(lu + 617), b[141], x);
      x = fma(-CHEM_LDLU(lu + 618), b[142], x);
      x = fma(-CHEM_LDLU(lu + 619), b[143], x);
      b[144] = x;
    }
}
__device__ __noinline__ void solve_s1_0_1(double* __restrict__ ws, int rhs)
{
    const double* __restrict__ lu = ws + 2426;
    const double* __restrict__ vd = ws + 4116;
    double* __restrict__ b = ws + rhs;
    (void)vd;
    {
      double x = b[145];
      x = fma(-CHEM_LDLU(lu + 620), b[32], x);
      x = fma(-CHEM_LDLU(lu + 621), b[38], x);
      x = fma(-CHEM_LDLU(lu + 622), b[40], x);
      x = fma(-CHEM_LDLU(lu + 623), b[42], x);
      x = fma(-CHEM_LDLU(lu + 624), b[51], x);
      x = fma(-CHEM_LDLU(lu + 625), b[53], x);
      x = fma(-CHEM_LDLU(lu + 626), b[55], x);
      x = fma(-CHEM_LDLU(lu + 627), b[58], x);
      x = fma(-CHEM_LDLU(lu + 628), b[61], x);
      x = fma(-CHEM_LDLU(lu + 629), b[63], x);
      x = fma(-CHEM_LDLU(lu + 630), b[64], x);
      x = fma(-CHEM_LDLU(lu + 631), b[66], x);
      x = fma(-CHEM_LDLU(lu + 632), b[68], x);
      x = fma(-CHEM_LDLU(lu + 633), b[73], x);
      x = fma(-CHEM_LDLU(lu + 634), b[74], x);
      x = fma(-CHEM_LDLU(lu + 635), b[75], x);
      x = fma(-CHEM_LDLU(lu + 636), b[76], x);
      x = fma(-CHEM_LDLU(lu + 637), b[79], x);
      x = fma(-CHEM_LDLU(lu + 638), b[83], x);
      x = fma(-CHEM_LDLU(lu + 639), b[89], x);
      x = fma(-CHEM_LDLU(lu + 640), b[93], x);
      x = fma(-CHEM_LDLU(lu + 641), b[98], x);
      x = fma(-CHEM_LDLU(lu + 642), b[104], x);
      x = fma(-CHEM_LDLU(lu + 643), b[107], x);
      x = fma(-CHEM_LDLU(lu + 644), b[110], x);
      x = fma(-CHEM_LDLU(lu + 645), b[111], x);
      x = fma(-CHEM_LDLU(lu + 646), b[113], x);
      x = fma(-CHEM_LDLU(lu + 647), b[119], x);
      x = fma(-CHEM_LDLU(lu + 648), b[120], x);
      x = fma(-CHEM_LDLU(lu + 649), b[121], x);
      x = fma(-CHEM_LDLU(lu + 650), b[123], x);
      x = fma(-CHEM_LDLU(lu + 651), b[125], x);
      x = fma(-CHEM_LDLU(lu + 652), b[127], x);
      x = fma(-CHEM_LDLU(lu + 653), b[128], x);
      x = fma(-CHEM_LDLU(lu + 654), b[129], x);
      x = fma(-CHEM_LDLU(lu + 655), b[130], x);
      x = fma(-CHEM_LDLU(lu + 656), b[131], x);
      x = fma(-CHEM_LDLU(lu + 657), b[132], x);
      x = fma(-CHEM_LDLU(lu + 658), b[133], x);
      x = fma(-CHEM_LDLU(lu + 659), b[134], x);
      x = fma(-CHEM_LDLU(lu + 660), b[135], x);
      x = fma(-CHEM_LDLU(lu + 661), b[136], x);
      x = fma(-CHEM_LDLU(lu + 662), b[137], x);
      x = fma(-CHEM_LDLU(lu + 663), b[138], x);
      x = fma(-CHEM_LDLU(lu + 664), b[139], x);
      x = fma(-CHEM_LDLU(lu + 665), b[141], x);
      x = fma(-CHEM_LDLU(lu + 666), b[142], x);
      x = fma(-CHEM_LDLU(lu + 667), b[143], x);
      x = fma(-CHEM_LDLU(lu + 668), b[144], x);
      b[145] = x;
    }
    {
      double x = b[146];
      x = fma(-CHEM_LDLU(lu + 669), b[10], x);
      x = fma(-CHEM_LDLU(lu + 670), b[12], x);
      x = fma(-CHEM_LDLU(lu + 671), b[13], x);
      x = fma(-CHEM_LDLU(lu + 672), b[26], x);
      x = fma(-CHEM_LDLU(lu + 673), b[27], x);
      x = fma(-CHEM_LDLU(lu + 674), b[28], x);
      x = fma(-CHEM_LDLU(lu + 675), b[29], x);
      x = fma(-CHEM_LDLU(lu + 676), b[30], x);
      x = fma(-CHEM_LDLU(lu + 677), b[33], x);
      x = fma(-CHEM_LDLU(lu + 678), b[34], x);
      x = fma(-CHEM_LDLU(lu + 679), b[35], x);
      x = fma(-CHEM_LDLU(lu + 680), b[36], x);
      x = fma(-CHEM_LDLU(lu + 681), b[42], x);
      x = fma(-CHEM_LDLU(lu + 682), b[51], x);
      x = fma(-CHEM_LDLU(lu + 683), b[52], x);
      x = fma(-CHEM_LDLU(lu + 684), b[61], x);
      x = fma(-CHEM_LDLU(lu + 685), b[62], x);
      x = fma(-CHEM_LDLU(lu + 686), b[64], x);
      x = fma(-CHEM_LDLU(lu + 687), b[66], x);
      x = fma(-CHEM_LDLU(lu + 688), b[71], x);
      x = fma(-CHEM_LDLU(lu + 689), b[79], x);
      x = fma(-CHEM_LDLU(lu + 690), b[83], x);
      x = fma(-CHEM_LDLU(lu + 691), b[89], x);
      x = fma(-CHEM_LDLU(lu + 692), b[90], x);
      x = fma(-CHEM_LDLU(lu + 693), b[97], x);
      x = fma(-CHEM_LDLU(lu + 694), b[98], x);
      x = fma(-CHEM_LDLU(lu + 695), b[103], x);
      x = fma(-CHEM_LDLU(lu + 696), b[106], x);
      x = fma(-CHEM_LDLU(lu + 697), b[107], x);
      x = fma(-CHEM_LDLU(lu + 698), b[109], x);
      x = fma(-CHEM_LDLU(lu + 699), b[111], x);
      x = fma(-CHEM_LDLU(lu + 700), b[112], x);
      x = fma(-CHEM_LDLU(lu + 701), b[113], x);
      x = fma(-CHEM_LDLU(lu + 702), b[117], x);
      x = fma(-CHEM_LDLU(lu + 703), b[119], x);
      x = fma(-CHEM_LDLU(lu + 704), b[120], x);
      x = fma(-CHEM_LDLU(lu + 705), b[121], x);
      x = fma(-CHEM_LDLU(lu + 706), b[122], x);
      x = fma(-CHEM_LDLU(lu + 707), b[123], x);
      x = fma(-CHEM_LDLU(lu + 708), b[125], x);
      x = fma(-CHEM_LDLU(lu + 709), b[127], x);
      x = fma(-CHEM_LDLU(lu + 710), b[128], x);
      x = fma(-CHEM_LDLU(lu + 711), b[129], x);
      x = fma(-CHEM_LDLU(lu + 712), b[130], x);
      x = fma(-CHEM_LDLU(lu + 713), b[132], x);
      x = fma(-CHEM_LDLU(lu + 714), b[133], x);
      x = fma(-CHEM_LDLU(lu + 715), b[134], x);
      x = fma(-CHEM_LDLU(lu + 716), b[135], x);
      x = fma(-CHEM_LDLU(lu + 717), b[136], x);
      x = fma(-CHEM_LDLU(lu + 718), b[137], x);
      x = fma(-CHEM_LDLU(lu + 719), b[138], x);
      x = fma(-CHEM_LDLU(lu + 720), b[139], x);
      x = fma(-CHEM_LDLU(lu + 721), b[141], x);
      x = fma(-CHEM_LDLU(lu + 722), b[142], x);
      x = fma(-CHEM_LDLU(lu + 723), b[143], x);
      x = fma(-CHEM_LDLU(lu + 724), b[144], x);
      x = fma(-CHEM_LDLU(lu + 725), b[145], x);
      b[146] = x;
    }
    {
      double x = b[147];
      x = fma(-CHEM_LDLU(lu + 726), b[11], x);
      x = fma(-CHEM_LDLU(lu + 727), b[12], x);
      x = fma(-CHEM_LDLU(lu + 728), b[27], x);
      x = fma(-CHEM_LDLU(lu + 729), b[30], x);
      x = fma(-CHEM_LDLU(lu + 730), b[34], x);
      x = fma(-CHEM_LDLU(lu + 731), b[35], x);
      x = fma(-CHEM_LDLU(lu + 732), b[36], x);
      x = fma(-CHEM_LDLU(lu + 733), b[53], x);
      x = fma(-CHEM_LDLU(lu + 734), b[54], x);
      x = fma(-CHEM_LDLU(lu + 735), b[55], x);
      x = fma(-CHEM_LDLU(lu + 736), b[62], x);
      x = fma(-CHEM_LDLU(lu + 737), b[67], x);
      x = fma(-CHEM_LDLU(lu + 738), b[68], x);
      x = fma(-CHEM_LDLU(lu + 739), b[69], x);
      x = fma(-CHEM_LDLU(lu + 740), b[78], x);
      x = fma(-CHEM_LDLU(lu + 741), b[79], x);
      x = fma(-CHEM_LDLU(lu + 742), b[80], x);
      x = fma(-CHEM_LDLU(lu + 743), b[83], x);
      x = fma(-CHEM_LDLU(lu + 744), b[85], x);
      x = fma(-CHEM_LDLU(lu + 745), b[89], x);
      x = fma(-CHEM_LDLU(lu + 746), b[90], x);
      x = fma(-CHEM_LDLU(lu + 747), b[92], x);
      x = fma(-CHEM_LDLU(lu + 748), b[97], x);
      x = fma(-CHEM_LDLU(lu + 749), b[98], x);
      x = fma(-CHEM_LDLU(lu + 750), b[101], x);
      x = fma(-CHEM_LDLU(lu + 751), b[103], x);
      x = fma(-CHEM_LDLU(lu + 752), b[104], x);
      x = fma(-CHEM_LDLU(lu + 753), b[107], x);
      x = fma(-CHEM_LDLU(lu + 754), b[108], x);
      x = fma(-CHEM_LDLU(lu + 755), b[109], x);
      x = fma(-CHEM_LDLU(lu + 756), b[110], x);
      x = fma(-CHEM_LDLU(lu + 757), b[111], x);
      x = fma(-CHEM_LDLU(lu + 758), b[112], x);
      x = fma(-CHEM_LDLU(lu + 759), b[113], x);
      x = fma(-CHEM_LDLU(lu + 760), b[117], x);
      x = fma(-CHEM_LDLU(lu + 761), b[118], x);
      x = fma(-CHEM_LDLU(lu + 762), b[119], x);
      x = fma(-CHEM_LDLU(lu + 763), b[120], x);
      x = fma(-CHEM_LDLU(lu + 764), b[121], x);
      x = fma(-CHEM_LDLU(lu + 765), b[123], x);
      x = fma(-CHEM_LDLU(lu + 766), b[125], x);
      x = fma(-CHEM_LDLU(lu + 767), b[127], x);
      x = fma(-CHEM_LDLU(lu + 768), b[128], x);
      x = fma(-CHEM_LDLU(lu + 769), b[129], x);
      x = fma(-CHEM_LDLU(lu + 770), b[130], x);
      x = fma(-CHEM_LDLU(lu + 771), b[132], x);
      x = fma(-CHEM_LDLU(lu + 772), b[133], x);
      x = fma(-CHEM_LDLU(lu + 773), b[134], x);
      x = fma(-CHEM_LDLU(lu + 774), b[135], x);
      x = fma(-CHEM_LDLU(lu + 775), b[136], x);
      x = fma(-CHEM_LDLU(lu + 776), b[137], x);
      x = fma(-CHEM_LDLU(lu + 777), b[138], x);
      x = fma(-CHEM_LDLU(lu + 778), b[139], x);
      x = fma(-CHEM_LDLU(lu + 779), b[140], x);
      x = fma(-CHEM_LDLU(lu + 780), b[141], x);
      x = fma(-CHEM_LDLU(lu + 781), b[142], x);
      x = fma(-CHEM_LDLU(lu + 782), b[143], x);
      x = fma(-CHEM_LDLU(lu + 783), b[144], x);
      x = fma(-CHEM_LDLU(lu + 784), b[145], x);
      x = fma(-CHEM_LDLU(lu + 785), b[146], x);
      b[147] = x;
    }
    {
      double x = b[148];
      x = fma(-CHEM_LDLU(lu + 786), b[11], x);
      x = fma(-CHEM_LDLU(lu + 787), b[12], x);
      x = fma(-CHEM_LDLU(lu + 788), b[13], x);
      x = fma(-CHEM_LDLU(lu + 789), b[14], x);
      x = fma(-CHEM_LDLU(lu + 790), b[21], x);
      x = fma(-CHEM_LDLU(lu + 791), b[22], x);
      x = fma(-CHEM_LDLU(lu + 792), b[23], x);
      x = fma(-CHEM_LDLU(lu + 793), b[24], x);
      x = fma(-CHEM_LDLU(lu + 794), b[26], x);
      x = fma(-CHEM_LDLU(lu + 795), b[27], x);
      x = fma(-CHEM_LDLU(lu + 796), b[28], x);
      x = fma(-CHEM_LDLU(lu + 797), b[32], x);
      x = fma(-CHEM_LDLU(lu + 798), b[33], x);
      x = fma(-CHEM_LDLU(lu + 799), b[34], x);
      x = fma(-CHEM_LDLU(lu + 800), b[35], x);
      x = fma(-CHEM_LDLU(lu + 801), b[36], x);
      x = fma(-CHEM_LDLU(lu + 802), b[45], x);
      x = fma(-CHEM_LDLU(lu + 803), b[46], x);
      x = fma(-CHEM_LDLU(lu + 804), b[47], x);
      x = fma(-CHEM_LDLU(lu + 805), b[48], x);
      x = fma(-CHEM_LDLU(lu + 806), b[51], x);
      x = fma(-CHEM_LDLU(lu + 807), b[52], x);
      x = fma(-CHEM_LDLU(lu + 808), b[53], x);
      x = fma(-CHEM_LDLU(lu + 809), b[54], x);
      x = fma(-CHEM_LDLU(lu + 810), b[55], x);
      x = fma(-CHEM_LDLU(lu + 811), b[56], x);
      x = fma(-CHEM_LDLU(lu + 812), b[57], x);
      x = fma(-CHEM_LDLU(lu + 813), b[58], x);
      x = fma(-CHEM_LDLU(lu + 814), b[61], x);
      x = fma(-CHEM_LDLU(lu + 815), b[63], x);
      x = fma(-CHEM_LDLU(lu + 816), b[64], x);
      x = fma(-CHEM_LDLU(lu + 817), b[66], x);
      x = fma(-CHEM_LDLU(lu + 818), b[68], x);
      x = fma(-CHEM_LDLU(lu + 819), b[69], x);
      x = fma(-CHEM_LDLU(lu + 820), b[71], x);
      x = fma(-CHEM_LDLU(lu + 821), b[72], x);
      x = fma(-CHEM_LDLU(lu + 822), b[73], x);
      x = fma(-CHEM_LDLU(lu + 823), b[74], x);
      x = fma(-CHEM_LDLU(lu + 824), b[75], x);
      x = fma(-CHEM_LDLU(lu + 825), b[76], x);
      x = fma(-CHEM_LDLU(lu + 826), b[77], x);
      x = fma(-CHEM_LDLU(lu + 827), b[79], x);
      x = fma(-CHEM_LDLU(lu + 828), b[83], x);
      x = fma(-CHEM_LDLU(lu + 829), b[84], x);
      x = fma(-CHEM_LDLU(lu + 830), b[85], x);
      x = fma(-CHEM_LDLU(lu + 831), b[86], x);
      x = fma(-CHEM_LDLU(lu + 832), b[87], x);
      x = fma(-CHEM_LDLU(lu + 833), b[88], x);
      x = fma(-CHEM_LDLU(lu + 834), b[90], x);
      x = fma(-CHEM_LDLU(lu + 835), b[91], x);
      x = fma(-CHEM_LDLU(lu + 836), b[93], x);
      x = fma(-CHEM_LDLU(lu + 837), b[94], x);
      x = fma(-CHEM_LDLU(lu + 838), b[98], x);
      x = fma(-CHEM_LDLU(lu + 839), b[99], x);
      x = fma(-CHEM_LDLU(lu + 840), b[100], x);
      x = fma(-CHEM_LDLU(lu + 841), b[101], x);
      x = fma(-CHEM_LDLU(lu + 842), b[103], x);
      x = fma(-CHEM_LDLU(lu + 843), b[104], x);
      x = fma(-CHEM_LDLU(lu + 844), b[105], x);
      x = fma(-CHEM_LDLU(lu + 845), b[106], x);
      x = fma(-CHEM_LDLU(lu + 846), b[107], x);
      x = fma(-CHEM_LDLU(lu + 847), b[108], x);
      x = fma(-CHEM_LDLU(lu + 848), b[110], x);
      x = fma(-CHEM_LDLU(lu + 849), b[111], x);
      x = fma(-CHEM_LDLU(lu + 850), b[113], x);
      x = fma(-CHEM_LDLU(lu + 851), b[114], x);
      x = fma(-CHEM_LDLU(lu + 852), b[115], x);
      x = fma(-CHEM_LDLU(lu + 853), b[116], x);
      x = fma(-CHEM_LDLU(lu + 854), b[117], x);
      x = fma(-CHEM_LDLU(lu + 855), b[118], x);
      x = fma(-CHEM_LDLU(lu + 856), b[119], x);
      x = fma(-CHEM_LDLU(lu + 857), b[120], x);
      x = fma(-CHEM_LDLU(lu + 858), b[121], x);
      x = fma(-CHEM_LDLU(lu + 859), b[122], x);
      x = fma(-CHEM_LDLU(lu + 860), b[123], x);
      x = fma(-CHEM_LDLU(lu + 861), b[124], x);
      x = fma(-CHEM_LDLU(lu + 862), b[125], x);
      x = fma(-CHEM_LDLU(lu + 863), b[127], x);
      x = fma(-CHEM_LDLU(lu + 864), b[128], x);
      x = fma(-CHEM_LDLU(lu + 865), b[129], x);
      x = fma(-CHEM_LDLU(lu + 866), b[130], x);
      x = fma(-CHEM_LDLU(lu + 867), b[131], x);
      x = fma(-CHEM_LDLU(lu + 868), b[132], x);
      x = fma(-CHEM_LDLU(lu + 869), b[133], x);
      x = fma(-CHEM_LDLU(lu + 870), b[134], x);
      x = fma(-CHEM_LDLU(lu + 871), b[135], x);
      x = fma(-CHEM_LDLU(lu + 872), b[136], x);
      x = fma(-CHEM_LDLU(lu + 873), b[137], x);
      x = fma(-CHEM_LDLU(lu + 874), b[138], x);
      x = fma(-CHEM_LDLU(lu + 875), b[139], x);
      x = fma(-CHEM_LDLU(lu + 876), b[140], x);
      x = fma(-CHEM_LDLU(lu + 877), b[141], x);
      x = fma(-CHEM_LDLU(lu + 878), b[142], x);
      x = fma(-CHEM_LDLU(lu + 879), b[143], x);
      x = fma(-CHEM_LDLU(lu + 880), b[144], x);
      x = fma(-CHEM_LDLU(lu + 881), b[145], x);
      x = fma(-CHEM_LDLU(lu + 882), b[146], x);
      x = fma(-CHEM_LDLU(lu + 883), b[147], x);
      b[148] = x;
    }
    {
      double x = b[148];
      b[148] = x * CHEM_LDLU(vd + 148);
    }
    {
      double x = b[147];
      x = fma(-CHEM_LDLU(lu + 884), b[148], x);
      b[147] = x * CHEM_LDLU(vd + 147);
    }
    {
      double x = b[146];
      x = fma(-CHEM_LDLU(lu + 885), b[147], x);
      x = fma(-CHEM_LDLU(lu + 886), b[148], x);
      b[146] = x * CHEM_LDLU(vd + 146);
    }
    {
      double x = b[145];
      x = fma(-CHEM_LDLU(lu + 887), b[146], x);
      x = fma(-CHEM_LDLU(lu + 888), b[147], x);
      x = fma(-CHEM_LDLU(lu + 889), b[148], x);
      b[145] = x * CHEM_LDLU(vd + 145);
    }
    {
      double x = b[144];
      x = fma(-CHEM_LDLU(lu + 890), b[145], x);
      x = fma(-CHEM_LDLU(lu + 891), b[146], x);
      x = fma(-CHEM_LDLU(lu + 892), b[147], x);
      x = fma(-CHEM_LDLU(lu + 893), b[148], x);
      b[144] = x * CHEM_LDLU(vd + 144);
    }
    {
      double x = b[143];
      x = fma(-CHEM_LDLU(lu + 894), b[144], x);
      x = fma(-CHEM_LDLU(lu + 895), b[145], x);
      x = fma(-CHEM_LDLU(lu + 896), b[146], x);
      x = fma(-CHEM_LDLU(lu + 897), b[147], x);
      x = fma(-CHEM_LDLU(lu + 898), b[148], x);
      b[143] = x * CHEM_LDLU(vd + 143);
    }
    {
      double x = b[142];
      x = fma(-CHEM_LDLU(lu + 899), b[143], x);
      x = fma(-CHEM_LDLU(lu + 900), b[144], x);
      x = fma(-CHEM_LDLU(lu + 901), b[145], x);
      x = fma(-CHEM_LDLU(lu + 902), b[146], x);
      x = fma(-CHEM_LDLU(lu + 903), b[147], x);
      x = fma(-CHEM_LDLU(lu + 904), b[148], x);
      b[142] = x * CHEM_LDLU(vd + 142);
    }
    {
      double x = b[141];
      x = fma(-CHEM_LDLU(lu + 905), b[142], x);
      x = fma(-CHEM_LDLU(lu + 906), b[143], x);
      x = fma(-CHEM_LDLU(lu + 907), b[144], x);
      x = fma(-CHEM_LDLU(lu + 908), b[145], x);
      x = fma(-CHEM_LDLU(lu + 909), b[146], x);
      x = fma(-CHEM_LDLU(lu + 910), b[147], x);
      x = fma(-CHEM_LDLU(lu + 911), b[148], x);
      b[141] = x * CHEM_LDLU(vd + 141);
    }
    {
      double x = b[140];
      x = fma(-CHEM_LDLU(lu + 912), b[141], x);
      x = fma(-CHEM_LDLU(lu + 913), b[142], x);
      x = fma(-CHEM_LDLU(lu + 914), b[143], x);
      x = fma(-CHEM_LDLU(lu + 915), b[144], x);
      x = fma(-CHEM_LDLU(lu + 916), b[145], x);
      x = fma(-CHEM_LDLU(lu + 917), b[146], x);
      x = fma(-CHEM_LDLU(lu + 918), b[147], x);
      x = fma(-CHEM_LDLU(lu + 919), b[148], x);
      b[140] = x * CHEM_LDLU(vd + 140);
    }
    {
      double x = b[139];
      x = fma(-CHEM_LDLU(lu + 920), b[141], x);
      x = fma(-CHEM_LDLU(lu + 921), b[142], x);
      x = fma(-CHEM_LDLU(lu + 922), b[143], x);
      x = fma(-CHEM_LDLU(lu + 923), b[144], x);
      x = fma(-CHEM_LDLU(lu + 924), b[145], x);
      x = fma(-CHEM_LDLU(lu + 925), b[146], x);
      x = fma(-CHEM_LDLU(lu + 926), b[147], x);
      x = fma(-CHEM_LDLU(lu + 927), b[148], x);
      b[139] = x * CHEM_LDLU(vd + 139);
    }
    {
      double x = b[138];
      x = fma(-CHEM_LDLU(lu + 928), b[139], x);
      x = fma(-CHEM_LDLU(lu + 929), b[141], x);
      x = fma(-CHEM_LDLU(lu + 930), b[142], x);
      x = fma(-CHEM_LDLU(lu + 931), b[143], x);
      x = fma(-CHEM_LDLU(lu + 932), b[144], x);
      x = fma(-CHEM_LDLU(lu + 933), b[145], x);
      x = fma(-CHEM_LDLU(lu + 934), b[146], x);
      x = fma(-CHEM_LDLU(lu + 935), b[147], x);
      x = fma(-CHEM_LDLU(lu + 936), b[148], x);
      b[138] = x * CHEM_LDLU(vd + 138);
    }
    {
      double x = b[137];
      x = fma(-CHEM_LDLU(lu + 937), b[138], x);
      x = fma(-CHEM_LDLU(lu + 938), b[139], x);
      x = fma(-CHEM_LDLU(lu + 939), b[141], x);
      x = fma(-CHEM_LDLU(lu + 940), b[142], x);
      x = fma(-CHEM_LDLU(lu + 941), b[143], x);
      x = fma(-CHEM_LDLU(lu + 942), b[144], x);
      x = fma(-CHEM_LDLU(lu + 943), b[145], x);
      x = fma(-CHEM_LDLU(lu + 944), b[146], x);
      x = fma(-CHEM_LDLU(lu + 945), b[147], x);
      x = fma(-CHEM_LDLU(lu + 946), b[148], x);
      b[137] = x * CHEM_LDLU(vd + 137);
    }
    {
      double x = b[136];
      x = fma(-CHEM_LDLU(lu + 947), b[137], x);
      x = fma(-CHEM_LDLU(lu + 948), b[138], x);
      x = fma(-CHEM_LDLU(lu + 949), b[139], x);
      x = fma(-CHEM_LDLU(lu + 950), b[141], x);
      x = fma(-CHEM_LDLU(lu + 951), b[142], x);
      x = fma(-CHEM_LDLU(lu + 952), b[144], x);
      x = fma(-CHEM_LDLU(lu + 953), b[145], x);
      x = fma(-CHEM_LDLU(lu + 954), b[146], x);
      x = fma(-CHEM_LDLU(lu + 955), b[147], x);
      x = fma(-CHEM_LDLU(lu + 956), b[148], x);
      b[136] = x * CHEM_LDLU(vd + 136);
    }
    {
      double x = b[135];
      x = fma(-CHEM_LDLU(lu + 957), b[137], x);
      x = fma(-CHEM_LDLU(lu + 958), b[138], x);
      x = fma(-CHEM_LDLU(lu + 959), b[139], x);
      x = fma(-CHEM_LDLU(lu + 960), b[141], x);
      x = fma(-CHEM_LDLU(lu + 961), b[142], x);
      x = fma(-CHEM_LDLU(lu + 962), b[144], x);
      x = fma(-CHEM_LDLU(lu + 963), b[145], x);
      x = fma(-CHEM_LDLU(lu + 964), b[146], x);
      x = fma(-CHEM_LDLU(lu + 965), b[147], x);
      x = fma(-CHEM_LDLU(lu + 966), b[148], x);
      b[135] = x * CHEM_LDLU(vd + 135);
    }
    {
      double x = b[134];
      x = fma(-CHEM_LDLU(lu + 967), b[135], x);
      x = fma(-CHEM_LDLU(lu + 968), b[136], x);
      x = fma(-CHEM_LDLU(lu + 969), b[137], x);
      x = fma(-CHEM_LDLU(lu + 970), b[138], x);
      x = fma(-CHEM_LDLU(lu + 971), b[139], x);
      x = fma(-CHEM_LDLU(lu + 972), b[141], x);
      x = fma(-CHEM_LDLU(lu + 973), b[142], x);
      x = fma(-CHEM_LDLU(lu + 974), b[143], x);
      x = fma(-CHEM_LDLU(lu + 975), b[144], x);
      x = fma(-CHEM_LDLU(lu + 976), b[145], x);
      x = fma(-CHEM_LDLU(lu + 977), b[146], x);
      x = fma(-CHEM_LDLU(lu + 978), b[147], x);
      x = fma(-CHEM_LDLU(lu + 979), b[148], x);
      b[134] = x * CHEM_LDLU(vd + 134);
    }
    {
      double x = b[133];
      x = fma(-CHEM_LDLU(lu + 980), b[135], x);
      x = fma(-CHEM_LDLU(lu + 981), b[137], x);
      x = fma(-CHEM_LDLU(lu + 982), b[138], x);
      x = fma(-CHEM_LDLU(lu + 983), b[139], x);
      x = fma(-CHEM_LDLU(lu + 984), b[141], x);
      x = fma(-CHEM_LDLU(lu + 985), b[142], x);
      x = fma(-CHEM_LDLU(lu + 986), b[144], x);
      x = fma(-CHEM_LDLU(lu + 987), b[145], x);
      x = fma(-CHEM_LDLU(lu + 988), b[146], x);
      x = fma(-CHEM_LDLU(lu + 989), b[147], x);
      x = fma(-CHEM_LDLU(lu + 990), b[148], x);
      b[133] = x * CHEM_LDLU(vd + 133);
    }
    {
      double x = b[132];
      x = fma(-CHEM_LDLU(lu + 991), b[135], x);
      x = fma(-CHEM_LDLU(lu + 992), b[137], x);
      x = fma(-CHEM_LDLU(lu + 993), b[138], x);
      x = fma(-CHEM_LDLU(lu + 994), b[139], x);
      x = fma(-CHEM_LDLU(lu + 995), b[141], x);
      x = fma(-CHEM_LDLU(lu + 996), b[142], x);
      x = fma(-CHEM_LDLU(lu + 997), b[144], x);
      x = fma(-CHEM_LDLU(lu + 998), b[145], x);
      x = fma(-CHEM_LDLU(lu + 999), b[146], x);
      x = fma(-CHEM_LDLU(lu + 1000), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1001), b[148], x);
      b[132] = x * CHEM_LDLU(vd + 132);
    }
    {
      double x = b[131];
      x = fma(-CHEM_LDLU(lu + 1002), b[132], x);
      x = fma(-CHEM_LDLU(lu + 1003), b[133], x);
      x = fma(-CHEM_LDLU(lu + 1004), b[134], x);
      x = fma(-CHEM_LDLU(lu + 1005), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1006), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1007), b[138], x);
      x = fma(-CHEM_LDLU(lu + 1008), b[139], x);
      x = fma(-CHEM_LDLU(lu + 1009), b[141], x);
      x = fma(-CHEM_LDLU(lu + 1010), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1011), b[144], x);
      x = fma(-CHEM_LDLU(lu + 1012), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1013), b[146], x);
      x = fma(-CHEM_LDLU(lu + 1014), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1015), b[148], x);
      b[131] = x * CHEM_LDLU(vd + 131);
    }
    {
      double x = b[130];
      x = fma(-CHEM_LDLU(lu + 1016), b[132], x);
      x = fma(-CHEM_LDLU(lu + 1017), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1018), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1019), b[138], x);
      x = fma(-CHEM_LDLU(lu + 1020), b[139], x);
      x = fma(-CHEM_LDLU(lu + 1021), b[141], x);
      x = fma(-CHEM_LDLU(lu + 1022), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1023), b[144], x);
      x = fma(-CHEM_LDLU(lu + 1024), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1025), b[146], x);
      x = fma(-CHEM_LDLU(lu + 1026), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1027), b[148], x);
      b[130] = x * CHEM_LDLU(vd + 130);
    }
    {
      double x = b[129];
      x = fma(-CHEM_LDLU(lu + 1028), b[130], x);
      x = fma(-CHEM_LDLU(lu + 1029), b[132], x);
      x = fma(-CHEM_LDLU(lu + 1030), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1031), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1032), b[139], x);
      x = fma(-CHEM_LDLU(lu + 1033), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1034), b[144], x);
      x = fma(-CHEM_LDLU(lu + 1035), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1036), b[146], x);
      x = fma(-CHEM_LDLU(lu + 1037), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1038), b[148], x);
      b[129] = x * CHEM_LDLU(vd + 129);
    }
    {
      double x = b[128];
      x = fma(-CHEM_LDLU(lu + 1039), b[130], x);
      x = fma(-CHEM_LDLU(lu + 1040), b[132], x);
      x = fma(-CHEM_LDLU(lu + 1041), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1042), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1043), b[139], x);
      x = fma(-CHEM_LDLU(lu + 1044), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1045), b[144], x);
      x = fma(-CHEM_LDLU(lu + 1046), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1047), b[146], x);
      x = fma(-CHEM_LDLU(lu + 1048), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1049), b[148], x);
      b[128] = x * CHEM_LDLU(vd + 128);
    }
    {
      double x = b[127];
      x = fma(-CHEM_LDLU(lu + 1050), b[130], x);
      x = fma(-CHEM_LDLU(lu + 1051), b[132], x);
      x = fma(-CHEM_LDLU(lu + 1052), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1053), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1054), b[139], x);
      x = fma(-CHEM_LDLU(lu + 1055), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1056), b[144], x);
      x = fma(-CHEM_LDLU(lu + 1057), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1058), b[146], x);
      x = fma(-CHEM_LDLU(lu + 1059), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1060), b[148], x);
      b[127] = x * CHEM_LDLU(vd + 127);
    }
    {
      double x = b[126];
      x = fma(-CHEM_LDLU(lu + 1061), b[130], x);
      x = fma(-CHEM_LDLU(lu + 1062), b[132], x);
      x = fma(-CHEM_LDLU(lu + 1063), b[134], x);
      x = fma(-CHEM_LDLU(lu + 1064), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1065), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1066), b[139], x);
      x = fma(-CHEM_LDLU(lu + 1067), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1068), b[144], x);
      x = fma(-CHEM_LDLU(lu + 1069), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1070), b[146], x);
      x = fma(-CHEM_LDLU(lu + 1071), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1072), b[148], x);
      b[126] = x * CHEM_LDLU(vd + 126);
    }
    {
      double x = b[125];
      x = fma(-CHEM_LDLU(lu + 1073), b[130], x);
      x = fma(-CHEM_LDLU(lu + 1074), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1075), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1076), b[139], x);
      x = fma(-CHEM_LDLU(lu + 1077), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1078), b[144], x);
      x = fma(-CHEM_LDLU(lu + 1079), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1080), b[146], x);
      x = fma(-CHEM_LDLU(lu + 1081), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1082), b[148], x);
      b[125] = x * CHEM_LDLU(vd + 125);
    }
    {
      double x = b[124];
      x = fma(-CHEM_LDLU(lu + 1083), b[127], x);
      x = fma(-CHEM_LDLU(lu + 1084), b[129], x);
      x = fma(-CHEM_LDLU(lu + 1085), b[130], x);
      x = fma(-CHEM_LDLU(lu + 1086), b[132], x);
      x = fma(-CHEM_LDLU(lu + 1087), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1088), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1089), b[138], x);
      x = fma(-CHEM_LDLU(lu + 1090), b[139], x);
      x = fma(-CHEM_LDLU(lu + 1091), b[141], x);
      x = fma(-CHEM_LDLU(lu + 1092), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1093), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1094), b[146], x);
      x = fma(-CHEM_LDLU(lu + 1095), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1096), b[148], x);
      b[124] = x * CHEM_LDLU(vd + 124);
    }
    {
      double x = b[123];
      x = fma(-CHEM_LDLU(lu + 1097), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1098), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1099), b[139], x);
      x = fma(-CHEM_LDLU(lu + 1100), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1101), b[144], x);
      x = fma(-CHEM_LDLU(lu + 1102), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1103), b[146], x);
      x = fma(-CHEM_LDLU(lu + 1104), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1105), b[148], x);
      b[123] = x * CHEM_LDLU(vd + 123);
    }
    {
      double x = b[122];
      x = fma(-CHEM_LDLU(lu + 1106), b[123], x);
      x = fma(-CHEM_LDLU(lu + 1107), b[128], x);
      x = fma(-CHEM_LDLU(lu + 1108), b[130], x);
      x = fma(-CHEM_LDLU(lu + 1109), b[134], x);
      x = fma(-CHEM_LDLU(lu + 1110), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1111), b[136], x);
      x = fma(-CHEM_LDLU(lu + 1112), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1113), b[138], x);
      x = fma(-CHEM_LDLU(lu + 1114), b[139], x);
      x = fma(-CHEM_LDLU(lu + 1115), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1116), b[143], x);
      x = fma(-CHEM_LDLU(lu + 1117), b[144], x);
      x = fma(-CHEM_LDLU(lu + 1118), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1119), b[146], x);
      x = fma(-CHEM_LDLU(lu + 1120), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1121), b[148], x);
      b[122] = x * CHEM_LDLU(vd + 122);
    }
    {
      double x = b[121];
      x = fma(-CHEM_LDLU(lu + 1122), b[130], x);
      x = fma(-CHEM_LDLU(lu + 1123), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1124), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1125), b[139], x);
      x = fma(-CHEM_LDLU(lu + 1126), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1127), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1128), b[146], x);
      x = fma(-CHEM_LDLU(lu + 1129), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1130), b[148], x);
      b[121] = x * CHEM_LDLU(vd + 121);
    }
    {
      double x = b[120];
      x = fma(-CHEM_LDLU(lu + 1131), b[121], x);
      x = fma(-CHEM_LDLU(lu + 1132), b[130], x);
      x = fma(-CHEM_LDLU(lu + 1133), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1134), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1135), b[139], x);
      x = fma(-CHEM_LDLU(lu + 1136), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1137), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1138), b[146], x);
      x = fma(-CHEM_LDLU(lu + 1139), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1140), b[148], x);
      b[120] = x * CHEM_LDLU(vd + 120);
    }
    {
      double x = b[119];
      x = fma(-CHEM_LDLU(lu + 1141), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1142), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1143), b[139], x);
      x = fma(-CHEM_LDLU(lu + 1144), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1145), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1146), b[146], x);
      x = fma(-CHEM_LDLU(lu + 1147), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1148), b[148], x);
      b[119] = x * CHEM_LDLU(vd + 119);
    }
    {
      double x = b[118];
      x = fma(-CHEM_LDLU(lu + 1149), b[121], x);
      x = fma(-CHEM_LDLU(lu + 1150), b[130], x);
      x = fma(-CHEM_LDLU(lu + 1151), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1152), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1153), b[139], x);
      x = fma(-CHEM_LDLU(lu + 1154), b[141], x);
      x = fma(-CHEM_LDLU(lu + 1155), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1156), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1157), b[146], x);
      x = fma(-CHEM_LDLU(lu + 1158), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1159), b[148], x);
      b[118] = x * CHEM_LDLU(vd + 118);
    }
    {
      double x = b[117];
      x = fma(-CHEM_LDLU(lu + 1160), b[121], x);
      x = fma(-CHEM_LDLU(lu + 1161), b[123], x);
      x = fma(-CHEM_LDLU(lu + 1162), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1163), b[139], x);
      x = fma(-CHEM_LDLU(lu + 1164), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1165), b[144], x);
      x = fma(-CHEM_LDLU(lu + 1166), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1167), b[146], x);
      x = fma(-CHEM_LDLU(lu + 1168), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1169), b[148], x);
      b[117] = x * CHEM_LDLU(vd + 117);
    }
    {
      double x = b[116];
      x = fma(-CHEM_LDLU(lu + 1170), b[148], x);
      b[116] = x * CHEM_LDLU(vd + 116);
    }
    {
      double x = b[115];
      x = fma(-CHEM_LDLU(lu + 1171), b[116], x);
      x = fma(-CHEM_LDLU(lu + 1172), b[148], x);
      b[115] = x * CHEM_LDLU(vd + 115);
    }
    {
      double x = b[114];
      x = fma(-CHEM_LDLU(lu + 1173), b[121], x);
      x = fma(-CHEM_LDLU(lu + 1174), b[130], x);
      x = fma(-CHEM_LDLU(lu + 1175), b[132], x);
      x = fma(-CHEM_LDLU(lu + 1176), b[134], x);
      x = fma(-CHEM_LDLU(lu + 1177), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1178), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1179), b[139], x);
      x = fma(-CHEM_LDLU(lu + 1180), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1181), b[144], x);
      x = fma(-CHEM_LDLU(lu + 1182), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1183), b[146], x);
      x = fma(-CHEM_LDLU(lu + 1184), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1185), b[148], x);
      b[114] = x * CHEM_LDLU(vd + 114);
    }
    {
      double x = b[113];
      x = fma(-CHEM_LDLU(lu + 1186), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1187), b[144], x);
      x = fma(-CHEM_LDLU(lu + 1188), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1189), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1190), b[148], x);
      b[113] = x * CHEM_LDLU(vd + 113);
    }
    {
      double x = b[112];
      x = fma(-CHEM_LDLU(lu + 1191), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1192), b[139], x);
      x = fma(-CHEM_LDLU(lu + 1193), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1194), b[146], x);
      x = fma(-CHEM_LDLU(lu + 1195), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1196), b[148], x);
      b[112] = x * CHEM_LDLU(vd + 112);
    }
    {
      double x = b[111];
      x = fma(-CHEM_LDLU(lu + 1197), b[121], x);
      x = fma(-CHEM_LDLU(lu + 1198), b[130], x);
      x = fma(-CHEM_LDLU(lu + 1199), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1200), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1201), b[139], x);
      x = fma(-CHEM_LDLU(lu + 1202), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1203), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1204), b[146], x);
      x = fma(-CHEM_LDLU(lu + 1205), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1206), b[148], x);
      b[111] = x * CHEM_LDLU(vd + 111);
    }
    {
      double x = b[110];
      x = fma(-CHEM_LDLU(lu + 1207), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1208), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1209), b[138], x);
      x = fma(-CHEM_LDLU(lu + 1210), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1211), b[144], x);
      x = fma(-CHEM_LDLU(lu + 1212), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1213), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1214), b[148], x);
      b[110] = x * CHEM_LDLU(vd + 110);
    }
    {
      double x = b[109];
      x = fma(-CHEM_LDLU(lu + 1215), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1216), b[139], x);
      x = fma(-CHEM_LDLU(lu + 1217), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1218), b[146], x);
      x = fma(-CHEM_LDLU(lu + 1219), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1220), b[148], x);
      b[109] = x * CHEM_LDLU(vd + 109);
    }
    {
      double x = b[108];
      x = fma(-CHEM_LDLU(lu + 1221), b[110], x);
      x = fma(-CHEM_LDLU(lu + 1222), b[111], x);
      x = fma(-CHEM_LDLU(lu + 1223), b[130], x);
      x = fma(-CHEM_LDLU(lu + 1224), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1225), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1226), b[139], x);
      x = fma(-CHEM_LDLU(lu + 1227), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1228), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1229), b[146], x);
      x = fma(-CHEM_LDLU(lu + 1230), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1231), b[148], x);
      b[108] = x * CHEM_LDLU(vd + 108);
    }
    {
      double x = b[107];
      x = fma(-CHEM_LDLU(lu + 1232), b[130], x);
      x = fma(-CHEM_LDLU(lu + 1233), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1234), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1235), b[139], x);
      x = fma(-CHEM_LDLU(lu + 1236), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1237), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1238), b[146], x);
      x = fma(-CHEM_LDLU(lu + 1239), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1240), b[148], x);
      b[107] = x * CHEM_LDLU(vd + 107);
    }
    {
      double x = b[106];
      x = fma(-CHEM_LDLU(lu + 1241), b[121], x);
      x = fma(-CHEM_LDLU(lu + 1242), b[132], x);
      x = fma(-CHEM_LDLU(lu + 1243), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1244), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1245), b[144], x);
      x = fma(-CHEM_LDLU(lu + 1246), b[148], x);
      b[106] = x * CHEM_LDLU(vd + 106);
    }
    {
      double x = b[105];
      x = fma(-CHEM_LDLU(lu + 1247), b[130], x);
      x = fma(-CHEM_LDLU(lu + 1248), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1249), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1250), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1251), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1252), b[146], x);
      x = fma(-CHEM_LDLU(lu + 1253), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1254), b[148], x);
      b[105] = x * CHEM_LDLU(vd + 105);
    }
    {
      double x = b[104];
      x = fma(-CHEM_LDLU(lu + 1255), b[113], x);
      x = fma(-CHEM_LDLU(lu + 1256), b[144], x);
      x = fma(-CHEM_LDLU(lu + 1257), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1258), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1259), b[148], x);
      b[104] = x * CHEM_LDLU(vd + 104);
    }
    {
      double x = b[103];
      x = fma(-CHEM_LDLU(lu + 1260), b[107], x);
      x = fma(-CHEM_LDLU(lu + 1261), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1262), b[139], x);
      x = fma(-CHEM_LDLU(lu + 1263), b[146], x);
      x = fma(-CHEM_LDLU(lu + 1264), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1265), b[148], x);
      b[103] = x * CHEM_LDLU(vd + 103);
    }
    {
      double x = b[102];
      x = fma(-CHEM_LDLU(lu + 1266), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1267), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1268), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1269), b[148], x);
      b[102] = x * CHEM_LDLU(vd + 102);
    }
    {
      double x = b[101];
      x = fma(-CHEM_LDLU(lu + 1270), b[107], x);
      x = fma(-CHEM_LDLU(lu + 1271), b[111], x);
      x = fma(-CHEM_LDLU(lu + 1272), b[130], x);
      x = fma(-CHEM_LDLU(lu + 1273), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1274), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1275), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1276), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1277), b[148], x);
      b[101] = x * CHEM_LDLU(vd + 101);
    }
    {
      double x = b[100];
      x = fma(-CHEM_LDLU(lu + 1278), b[115], x);
      x = fma(-CHEM_LDLU(lu + 1279), b[116], x);
      x = fma(-CHEM_LDLU(lu + 1280), b[148], x);
      b[100] = x * CHEM_LDLU(vd + 100);
    }
    {
      double x = b[99];
      x = fma(-CHEM_LDLU(lu + 1281), b[100], x);
      x = fma(-CHEM_LDLU(lu + 1282), b[115], x);
      x = fma(-CHEM_LDLU(lu + 1283), b[116], x);
      x = fma(-CHEM_LDLU(lu + 1284), b[148], x);
      b[99] = x * CHEM_LDLU(vd + 99);
    }
    {
      double x = b[98];
      x = fma(-CHEM_LDLU(lu + 1285), b[107], x);
      x = fma(-CHEM_LDLU(lu + 1286), b[130], x);
      x = fma(-CHEM_LDLU(lu + 1287), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1288), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1289), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1290), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1291), b[148], x);
      b[98] = x * CHEM_LDLU(vd + 98);
    }
    {
      double x = b[97];
      x = fma(-CHEM_LDLU(lu + 1292), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1293), b[139], x);
      x = fma(-CHEM_LDLU(lu + 1294), b[146], x);
      x = fma(-CHEM_LDLU(lu + 1295), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1296), b[148], x);
      b[97] = x * CHEM_LDLU(vd + 97);
    }
    {
      double x = b[96];
      x = fma(-CHEM_LDLU(lu + 1297), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1298), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1299), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1300), b[148], x);
      b[96] = x * CHEM_LDLU(vd + 96);
    }
    {
      double x = b[95];
      x = fma(-CHEM_LDLU(lu + 1301), b[108], x);
      x = fma(-CHEM_LDLU(lu + 1302), b[110], x);
      x = fma(-CHEM_LDLU(lu + 1303), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1304), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1305), b[148], x);
      b[95] = x * CHEM_LDLU(vd + 95);
    }
    {
      double x = b[94];
      x = fma(-CHEM_LDLU(lu + 1306), b[108], x);
      x = fma(-CHEM_LDLU(lu + 1307), b[110], x);
      x = fma(-CHEM_LDLU(lu + 1308), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1309), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1310), b[148], x);
      b[94] = x * CHEM_LDLU(vd + 94);
    }
    {
      double x = b[93];
      x = fma(-CHEM_LDLU(lu + 1311), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1312), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1313), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1314), b[148], x);
      b[93] = x * CHEM_LDLU(vd + 93);
    }
    {
      double x = b[92];
      x = fma(-CHEM_LDLU(lu + 1315), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1316), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1317), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1318), b[148], x);
      b[92] = x * CHEM_LDLU(vd + 92);
    }
    {
      double x = b[91];
      x = fma(-CHEM_LDLU(lu + 1319), b[99], x);
      x = fma(-CHEM_LDLU(lu + 1320), b[100], x);
      x = fma(-CHEM_LDLU(lu + 1321), b[115], x);
      x = fma(-CHEM_LDLU(lu + 1322), b[116], x);
      x = fma(-CHEM_LDLU(lu + 1323), b[148], x);
      b[91] = x * CHEM_LDLU(vd + 91);
    }
    {
      double x = b[90];
      x = fma(-CHEM_LDLU(lu + 1324), b[134], x);
      x = fma(-CHEM_LDLU(lu + 1325), b[136], x);
      x = fma(-CHEM_LDLU(lu + 1326), b[143], x);
      x = fma(-CHEM_LDLU(lu + 1327), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1328), b[148], x);
      b[90] = x * CHEM_LDLU(vd + 90);
    }
    {
      double x = b[89];
      x = fma(-CHEM_LDLU(lu + 1329), b[130], x);
      x = fma(-CHEM_LDLU(lu + 1330), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1331), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1332), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1333), b[146], x);
      x = fma(-CHEM_LDLU(lu + 1334), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1335), b[148], x);
      b[89] = x * CHEM_LDLU(vd + 89);
    }
    {
      double x = b[88];
      x = fma(-CHEM_LDLU(lu + 1336), b[148], x);
      b[88] = x * CHEM_LDLU(vd + 88);
    }
    {
      double x = b[87];
      x = fma(-CHEM_LDLU(lu + 1337), b[88], x);
      x = fma(-CHEM_LDLU(lu + 1338), b[148], x);
      b[87] = x * CHEM_LDLU(vd + 87);
    }
    {
      double x = b[86];
      x = fma(-CHEM_LDLU(lu + 1339), b[87], x);
      x = fma(-CHEM_LDLU(lu + 1340), b[88], x);
      x = fma(-CHEM_LDLU(lu + 1341), b[148], x);
      b[86] = x * CHEM_LDLU(vd + 86);
    }
    {
      double x = b[85];
      x = fma(-CHEM_LDLU(lu + 1342), b[120], x);
      x = fma(-CHEM_LDLU(lu + 1343), b[138], x);
      x = fma(-CHEM_LDLU(lu + 1344), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1345), b[146], x);
      x = fma(-CHEM_LDLU(lu + 1346), b[148], x);
      b[85] = x * CHEM_LDLU(vd + 85);
    }
}
__device__ __noinline__ void solve_s1_0_2(double* __restrict__ ws, int rhs)
{
    const double* __restrict__ lu = ws + 2426;
    const double* __restrict__ vd = ws + 4116;
    double* __restrict__ b = ws + rhs;
    (void)vd;
    {
      double x = b[84];
      x = fma(-CHEM_LDLU(lu + 1347), b[117], x);
      x = fma(-CHEM_LDLU(lu + 1348), b[128], x);
      x = fma(-CHEM_LDLU(lu + 1349), b[139], x);
      x = fma(-CHEM_LDLU(lu + 1350), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1351), b[148], x);
      b[84] = x * CHEM_LDLU(vd + 84);
    }
    {
      double x = b[83];
      x = fma(-CHEM_LDLU(lu + 1352), b[130], x);
      x = fma(-CHEM_LDLU(lu + 1353), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1354), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1355), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1356), b[148], x);
      b[83] = x * CHEM_LDLU(vd + 83);
    }
    {
      double x = b[82];
      x = fma(-CHEM_LDLU(lu + 1357), b[92], x);
      x = fma(-CHEM_LDLU(lu + 1358), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1359), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1360), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1361), b[148], x);
      b[82] = x * CHEM_LDLU(vd + 82);
    }
    {
      double x = b[81];
      x = fma(-CHEM_LDLU(lu + 1362), b[144], x);
      x = fma(-CHEM_LDLU(lu + 1363), b[145], x);
      b[81] = x * CHEM_LDLU(vd + 81);
    }
    {
      double x = b[80];
      x = fma(-CHEM_LDLU(lu + 1364), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1365), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1366), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1367), b[148], x);
      b[80] = x * CHEM_LDLU(vd + 80);
    }
    {
      double x = b[79];
      x = fma(-CHEM_LDLU(lu + 1368), b[130], x);
      x = fma(-CHEM_LDLU(lu + 1369), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1370), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1371), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1372), b[148], x);
      b[79] = x * CHEM_LDLU(vd + 79);
    }
    {
      double x = b[78];
      x = fma(-CHEM_LDLU(lu + 1373), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1374), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1375), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1376), b[148], x);
      b[78] = x * CHEM_LDLU(vd + 78);
    }
    {
      double x = b[77];
      x = fma(-CHEM_LDLU(lu + 1377), b[104], x);
      x = fma(-CHEM_LDLU(lu + 1378), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1379), b[144], x);
      x = fma(-CHEM_LDLU(lu + 1380), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1381), b[148], x);
      b[77] = x * CHEM_LDLU(vd + 77);
    }
    {
      double x = b[76];
      x = fma(-CHEM_LDLU(lu + 1382), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1383), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1384), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1385), b[148], x);
      b[76] = x * CHEM_LDLU(vd + 76);
    }
    {
      double x = b[75];
      x = fma(-CHEM_LDLU(lu + 1386), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1387), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1388), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1389), b[148], x);
      b[75] = x * CHEM_LDLU(vd + 75);
    }
    {
      double x = b[74];
      x = fma(-CHEM_LDLU(lu + 1390), b[130], x);
      x = fma(-CHEM_LDLU(lu + 1391), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1392), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1393), b[148], x);
      b[74] = x * CHEM_LDLU(vd + 74);
    }
    {
      double x = b[73];
      x = fma(-CHEM_LDLU(lu + 1394), b[130], x);
      x = fma(-CHEM_LDLU(lu + 1395), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1396), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1397), b[148], x);
      b[73] = x * CHEM_LDLU(vd + 73);
    }
    {
      double x = b[72];
      x = fma(-CHEM_LDLU(lu + 1398), b[86], x);
      x = fma(-CHEM_LDLU(lu + 1399), b[87], x);
      x = fma(-CHEM_LDLU(lu + 1400), b[88], x);
      x = fma(-CHEM_LDLU(lu + 1401), b[148], x);
      b[72] = x * CHEM_LDLU(vd + 72);
    }
    {
      double x = b[71];
      x = fma(-CHEM_LDLU(lu + 1402), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1403), b[138], x);
      x = fma(-CHEM_LDLU(lu + 1404), b[141], x);
      x = fma(-CHEM_LDLU(lu + 1405), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1406), b[148], x);
      b[71] = x * CHEM_LDLU(vd + 71);
    }
    {
      double x = b[70];
      x = fma(-CHEM_LDLU(lu + 1407), b[78], x);
      x = fma(-CHEM_LDLU(lu + 1408), b[80], x);
      x = fma(-CHEM_LDLU(lu + 1409), b[92], x);
      x = fma(-CHEM_LDLU(lu + 1410), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1411), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1412), b[148], x);
      b[70] = x * CHEM_LDLU(vd + 70);
    }
    {
      double x = b[69];
      x = fma(-CHEM_LDLU(lu + 1413), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1414), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1415), b[148], x);
      b[69] = x * CHEM_LDLU(vd + 69);
    }
    {
      double x = b[68];
      x = fma(-CHEM_LDLU(lu + 1416), b[104], x);
      x = fma(-CHEM_LDLU(lu + 1417), b[144], x);
      x = fma(-CHEM_LDLU(lu + 1418), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1419), b[148], x);
      b[68] = x * CHEM_LDLU(vd + 68);
    }
    {
      double x = b[67];
      x = fma(-CHEM_LDLU(lu + 1420), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1421), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1422), b[148], x);
      b[67] = x * CHEM_LDLU(vd + 67);
    }
    {
      double x = b[66];
      x = fma(-CHEM_LDLU(lu + 1423), b[130], x);
      x = fma(-CHEM_LDLU(lu + 1424), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1425), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1426), b[148], x);
      b[66] = x * CHEM_LDLU(vd + 66);
    }
    {
      double x = b[65];
      x = fma(-CHEM_LDLU(lu + 1427), b[66], x);
      x = fma(-CHEM_LDLU(lu + 1428), b[130], x);
      x = fma(-CHEM_LDLU(lu + 1429), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1430), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1431), b[148], x);
      b[65] = x * CHEM_LDLU(vd + 65);
    }
    {
      double x = b[64];
      x = fma(-CHEM_LDLU(lu + 1432), b[130], x);
      x = fma(-CHEM_LDLU(lu + 1433), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1434), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1435), b[148], x);
      b[64] = x * CHEM_LDLU(vd + 64);
    }
    {
      double x = b[63];
      x = fma(-CHEM_LDLU(lu + 1436), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1437), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1438), b[148], x);
      b[63] = x * CHEM_LDLU(vd + 63);
    }
    {
      double x = b[62];
      x = fma(-CHEM_LDLU(lu + 1439), b[132], x);
      x = fma(-CHEM_LDLU(lu + 1440), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1441), b[148], x);
      b[62] = x * CHEM_LDLU(vd + 62);
    }
    {
      double x = b[61];
      x = fma(-CHEM_LDLU(lu + 1442), b[128], x);
      x = fma(-CHEM_LDLU(lu + 1443), b[144], x);
      x = fma(-CHEM_LDLU(lu + 1444), b[148], x);
      b[61] = x * CHEM_LDLU(vd + 61);
    }
    {
      double x = b[60];
      x = fma(-CHEM_LDLU(lu + 1445), b[144], x);
      x = fma(-CHEM_LDLU(lu + 1446), b[145], x);
      b[60] = x * CHEM_LDLU(vd + 60);
    }
    {
      double x = b[59];
      x = fma(-CHEM_LDLU(lu + 1447), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1448), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1449), b[148], x);
      b[59] = x * CHEM_LDLU(vd + 59);
    }
    {
      double x = b[58];
      x = fma(-CHEM_LDLU(lu + 1450), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1451), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1452), b[148], x);
      b[58] = x * CHEM_LDLU(vd + 58);
    }
    {
      double x = b[57];
      x = fma(-CHEM_LDLU(lu + 1453), b[110], x);
      x = fma(-CHEM_LDLU(lu + 1454), b[144], x);
      x = fma(-CHEM_LDLU(lu + 1455), b[147], x);
      b[57] = x * CHEM_LDLU(vd + 57);
    }
    {
      double x = b[56];
      x = fma(-CHEM_LDLU(lu + 1456), b[117], x);
      x = fma(-CHEM_LDLU(lu + 1457), b[144], x);
      x = fma(-CHEM_LDLU(lu + 1458), b[148], x);
      b[56] = x * CHEM_LDLU(vd + 56);
    }
    {
      double x = b[55];
      x = fma(-CHEM_LDLU(lu + 1459), b[113], x);
      x = fma(-CHEM_LDLU(lu + 1460), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1461), b[148], x);
      b[55] = x * CHEM_LDLU(vd + 55);
    }
    {
      double x = b[54];
      x = fma(-CHEM_LDLU(lu + 1462), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1463), b[141], x);
      x = fma(-CHEM_LDLU(lu + 1464), b[147], x);
      b[54] = x * CHEM_LDLU(vd + 54);
    }
    {
      double x = b[53];
      x = fma(-CHEM_LDLU(lu + 1465), b[144], x);
      x = fma(-CHEM_LDLU(lu + 1466), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1467), b[148], x);
      b[53] = x * CHEM_LDLU(vd + 53);
    }
    {
      double x = b[52];
      x = fma(-CHEM_LDLU(lu + 1468), b[107], x);
      x = fma(-CHEM_LDLU(lu + 1469), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1470), b[148], x);
      b[52] = x * CHEM_LDLU(vd + 52);
    }
    {
      double x = b[51];
      x = fma(-CHEM_LDLU(lu + 1471), b[107], x);
      x = fma(-CHEM_LDLU(lu + 1472), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1473), b[148], x);
      b[51] = x * CHEM_LDLU(vd + 51);
    }
    {
      double x = b[50];
      x = fma(-CHEM_LDLU(lu + 1474), b[63], x);
      x = fma(-CHEM_LDLU(lu + 1475), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1476), b[148], x);
      b[50] = x * CHEM_LDLU(vd + 50);
    }
    {
      double x = b[49];
      x = fma(-CHEM_LDLU(lu + 1477), b[94], x);
      x = fma(-CHEM_LDLU(lu + 1478), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1479), b[148], x);
      b[49] = x * CHEM_LDLU(vd + 49);
    }
    {
      double x = b[48];
      x = fma(-CHEM_LDLU(lu + 1480), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1481), b[148], x);
      b[48] = x * CHEM_LDLU(vd + 48);
    }
    {
      double x = b[47];
      x = fma(-CHEM_LDLU(lu + 1482), b[86], x);
      x = fma(-CHEM_LDLU(lu + 1483), b[148], x);
      b[47] = x * CHEM_LDLU(vd + 47);
    }
    {
      double x = b[46];
      x = fma(-CHEM_LDLU(lu + 1484), b[148], x);
      b[46] = x * CHEM_LDLU(vd + 46);
    }
    {
      double x = b[45];
      x = fma(-CHEM_LDLU(lu + 1485), b[148], x);
      b[45] = x * CHEM_LDLU(vd + 45);
    }
    {
      double x = b[44];
      b[44] = x * CHEM_LDLU(vd + 44);
    }
    {
      double x = b[43];
      b[43] = x * CHEM_LDLU(vd + 43);
    }
    {
      double x = b[42];
      x = fma(-CHEM_LDLU(lu + 1486), b[139], x);
      x = fma(-CHEM_LDLU(lu + 1487), b[144], x);
      b[42] = x * CHEM_LDLU(vd + 42);
    }
    {
      double x = b[41];
      x = fma(-CHEM_LDLU(lu + 1488), b[52], x);
      x = fma(-CHEM_LDLU(lu + 1489), b[148], x);
      b[41] = x * CHEM_LDLU(vd + 41);
    }
    {
      double x = b[40];
      x = fma(-CHEM_LDLU(lu + 1490), b[144], x);
      x = fma(-CHEM_LDLU(lu + 1491), b[145], x);
      b[40] = x * CHEM_LDLU(vd + 40);
    }
    {
      double x = b[39];
      x = fma(-CHEM_LDLU(lu + 1492), b[40], x);
      b[39] = x * CHEM_LDLU(vd + 39);
    }
    {
      double x = b[38];
      x = fma(-CHEM_LDLU(lu + 1493), b[110], x);
      x = fma(-CHEM_LDLU(lu + 1494), b[144], x);
      b[38] = x * CHEM_LDLU(vd + 38);
    }
    {
      double x = b[37];
      x = fma(-CHEM_LDLU(lu + 1495), b[94], x);
      x = fma(-CHEM_LDLU(lu + 1496), b[110], x);
      b[37] = x * CHEM_LDLU(vd + 37);
    }
    {
      double x = b[36];
      x = fma(-CHEM_LDLU(lu + 1497), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1498), b[148], x);
      b[36] = x * CHEM_LDLU(vd + 36);
    }
    {
      double x = b[35];
      x = fma(-CHEM_LDLU(lu + 1499), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1500), b[148], x);
      b[35] = x * CHEM_LDLU(vd + 35);
    }
    {
      double x = b[34];
      x = fma(-CHEM_LDLU(lu + 1501), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1502), b[148], x);
      b[34] = x * CHEM_LDLU(vd + 34);
    }
    {
      double x = b[33];
      x = fma(-CHEM_LDLU(lu + 1503), b[52], x);
      x = fma(-CHEM_LDLU(lu + 1504), b[148], x);
      b[33] = x * CHEM_LDLU(vd + 33);
    }
    {
      double x = b[32];
      x = fma(-CHEM_LDLU(lu + 1505), b[107], x);
      x = fma(-CHEM_LDLU(lu + 1506), b[145], x);
      b[32] = x * CHEM_LDLU(vd + 32);
    }
    {
      double x = b[31];
      x = fma(-CHEM_LDLU(lu + 1507), b[79], x);
      x = fma(-CHEM_LDLU(lu + 1508), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1509), b[148], x);
      b[31] = x * CHEM_LDLU(vd + 31);
    }
    {
      double x = b[30];
      x = fma(-CHEM_LDLU(lu + 1510), b[62], x);
      x = fma(-CHEM_LDLU(lu + 1511), b[144], x);
      b[30] = x * CHEM_LDLU(vd + 30);
    }
    {
      double x = b[29];
      x = fma(-CHEM_LDLU(lu + 1512), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1513), b[148], x);
      b[29] = x * CHEM_LDLU(vd + 29);
    }
    {
      double x = b[28];
      x = fma(-CHEM_LDLU(lu + 1514), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1515), b[148], x);
      b[28] = x * CHEM_LDLU(vd + 28);
    }
    {
      double x = b[27];
      x = fma(-CHEM_LDLU(lu + 1516), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1517), b[148], x);
      b[27] = x * CHEM_LDLU(vd + 27);
    }
    {
      double x = b[26];
      x = fma(-CHEM_LDLU(lu + 1518), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1519), b[148], x);
      b[26] = x * CHEM_LDLU(vd + 26);
    }
    {
      double x = b[25];
      x = fma(-CHEM_LDLU(lu + 1520), b[148], x);
      b[25] = x * CHEM_LDLU(vd + 25);
    }
    {
      double x = b[24];
      x = fma(-CHEM_LDLU(lu + 1521), b[148], x);
      b[24] = x * CHEM_LDLU(vd + 24);
    }
    {
      double x = b[23];
      x = fma(-CHEM_LDLU(lu + 1522), b[148], x);
      b[23] = x * CHEM_LDLU(vd + 23);
    }
    {
      double x = b[22];
      x = fma(-CHEM_LDLU(lu + 1523), b[148], x);
      b[22] = x * CHEM_LDLU(vd + 22);
    }
    {
      double x = b[21];
      x = fma(-CHEM_LDLU(lu + 1524), b[135], x);
      b[21] = x * CHEM_LDLU(vd + 21);
    }
    {
      double x = b[20];
      x = fma(-CHEM_LDLU(lu + 1525), b[125], x);
      x = fma(-CHEM_LDLU(lu + 1526), b[133], x);
      b[20] = x * CHEM_LDLU(vd + 20);
    }
    {
      double x = b[19];
      x = fma(-CHEM_LDLU(lu + 1527), b[41], x);
      b[19] = x * CHEM_LDLU(vd + 19);
    }
    {
      double x = b[18];
      x = fma(-CHEM_LDLU(lu + 1528), b[41], x);
      b[18] = x * CHEM_LDLU(vd + 18);
    }
    {
      double x = b[17];
      x = fma(-CHEM_LDLU(lu + 1529), b[39], x);
      b[17] = x * CHEM_LDLU(vd + 17);
    }
    {
      double x = b[16];
      x = fma(-CHEM_LDLU(lu + 1530), b[60], x);
      b[16] = x * CHEM_LDLU(vd + 16);
    }
    {
      double x = b[15];
      x = fma(-CHEM_LDLU(lu + 1531), b[60], x);
      b[15] = x * CHEM_LDLU(vd + 15);
    }
    {
      double x = b[14];
      x = fma(-CHEM_LDLU(lu + 1532), b[148], x);
      b[14] = x * CHEM_LDLU(vd + 14);
    }
    {
      double x = b[13];
      x = fma(-CHEM_LDLU(lu + 1533), b[148], x);
      b[13] = x * CHEM_LDLU(vd + 13);
    }
    {
      double x = b[12];
      x = fma(-CHEM_LDLU(lu + 1534), b[148], x);
      b[12] = x * CHEM_LDLU(vd + 12);
    }
    {
      double x = b[11];
      x = fma(-CHEM_LDLU(lu + 1535), b[148], x);
      b[11] = x * CHEM_LDLU(vd + 11);
    }
    {
      double x = b[10];
      x = fma(-CHEM_LDLU(lu + 1536), b[30], x);
      b[10] = x * CHEM_LDLU(vd + 10);
    }
    {
      double x = b[9];
      x = fma(-CHEM_LDLU(lu + 1537), b[69], x);
      x = fma(-CHEM_LDLU(lu + 1538), b[148], x);
      b[9] = x * CHEM_LDLU(vd + 9);
    }
    {
      double x = b[8];
      x = fma(-CHEM_LDLU(lu + 1539), b[69], x);
      x = fma(-CHEM_LDLU(lu + 1540), b[148], x);
      b[8] = x * CHEM_LDLU(vd + 8);
    }
    {
      double x = b[7];
      b[7] = x * CHEM_LDLU(vd + 7);
    }
    {
      double x = b[6];
      b[6] = x * CHEM_LDLU(vd + 6);
    }
    {
      double x = b[5];
      b[5] = x * CHEM_LDLU(vd + 5);
    }
    {
      double x = b[4];
      b[4] = x * CHEM_LDLU(vd + 4);
    }
    {
      double x = b[3];
      b[3] = x * CHEM_LDLU(vd + 3);
    }
    {
      double x = b[2];
      b[2] = x * CHEM_LDLU(vd + 2);
    }
    {
      double x = b[1];
      b[1] = x * CHEM_LDLU(vd + 1);
    }
    {
      double x = b[0];
      b[0] = x * CHEM_LDLU(vd + 0);
    }
}
}  // namespace mech_cb6r5_ae7_aq
