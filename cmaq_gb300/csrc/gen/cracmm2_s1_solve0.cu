// Generated by cmaq_gb300.mechgen.generate from CCTM/src/MECHS/cracmm2/RXNS_DATA_MODULE.F90
// and RXNS_FUNC_MODULE.F90 (sha256/16 61a0c9d4d7262bbb).  Do not edit.
#include "cracmm2_mech.cuh"
#include <math.h>
namespace mech_cracmm2 {
__device__ __noinline__ void solve_s1_0_0(double* __restrict__ ws, int rhs)
{
    const double* __restrict__ lu = ws + 3484;
    const double* __restrict__ vd = ws + 6769;
    double* __restrict__ b = ws + rhs;
    (void)vd;
    {
      double x = b[0];
      b[0] = x;
    }
    {
      double x = b[1];
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
      x = fma(-CHEM_LDLU(lu + 1), b[5], x);
      b[6] = x;
    }
    {
      double x = b[7];
      x = fma(-CHEM_LDLU(lu + 2), b[5], x);
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
      x = fma(-CHEM_LDLU(lu + 3), b[16], x);
      b[17] = x;
    }
    {
      double x = b[18];
      b[18] = x;
    }
    {
      double x = b[19];
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
      b[29] = x;
    }
    {
      double x = b[30];
      x = fma(-CHEM_LDLU(lu + 4), b[3], x);
      x = fma(-CHEM_LDLU(lu + 5), b[4], x);
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
      x = fma(-CHEM_LDLU(lu + 6), b[16], x);
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
      x = fma(-CHEM_LDLU(lu + 7), b[38], x);
      b[39] = x;
    }
    {
      double x = b[40];
      b[40] = x;
    }
    {
      double x = b[41];
      b[41] = x;
    }
    {
      double x = b[42];
      b[42] = x;
    }
    {
      double x = b[43];
      x = fma(-CHEM_LDLU(lu + 8), b[42], x);
      b[43] = x;
    }
    {
      double x = b[44];
      b[44] = x;
    }
    {
      double x = b[45];
      b[45] = x;
    }
    {
      double x = b[46];
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
      x = fma(-CHEM_LDLU(lu + 9), b[41], x);
      b[51] = x;
    }
    {
      double x = b[52];
      x = fma(-CHEM_LDLU(lu + 10), b[42], x);
      x = fma(-CHEM_LDLU(lu + 11), b[51], x);
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
      x = fma(-CHEM_LDLU(lu + 12), b[39], x);
      b[55] = x;
    }
    {
      double x = b[56];
      b[56] = x;
    }
    {
      double x = b[57];
      b[57] = x;
    }
    {
      double x = b[58];
      b[58] = x;
    }
    {
      double x = b[59];
      x = fma(-CHEM_LDLU(lu + 13), b[36], x);
      b[59] = x;
    }
    {
      double x = b[60];
      x = fma(-CHEM_LDLU(lu + 14), b[50], x);
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
      b[65] = x;
    }
    {
      double x = b[66];
      b[66] = x;
    }
    {
      double x = b[67];
      b[67] = x;
    }
    {
      double x = b[68];
      x = fma(-CHEM_LDLU(lu + 15), b[36], x);
      x = fma(-CHEM_LDLU(lu + 16), b[44], x);
      b[68] = x;
    }
    {
      double x = b[69];
      x = fma(-CHEM_LDLU(lu + 17), b[51], x);
      b[69] = x;
    }
    {
      double x = b[70];
      x = fma(-CHEM_LDLU(lu + 18), b[49], x);
      b[70] = x;
    }
    {
      double x = b[71];
      b[71] = x;
    }
    {
      double x = b[72];
      x = fma(-CHEM_LDLU(lu + 19), b[50], x);
      b[72] = x;
    }
    {
      double x = b[73];
      x = fma(-CHEM_LDLU(lu + 20), b[18], x);
      b[73] = x;
    }
    {
      double x = b[74];
      x = fma(-CHEM_LDLU(lu + 21), b[19], x);
      b[74] = x;
    }
    {
      double x = b[75];
      x = fma(-CHEM_LDLU(lu + 22), b[20], x);
      b[75] = x;
    }
    {
      double x = b[76];
      x = fma(-CHEM_LDLU(lu + 23), b[21], x);
      b[76] = x;
    }
    {
      double x = b[77];
      x = fma(-CHEM_LDLU(lu + 24), b[22], x);
      b[77] = x;
    }
    {
      double x = b[78];
      x = fma(-CHEM_LDLU(lu + 25), b[23], x);
      b[78] = x;
    }
    {
      double x = b[79];
      x = fma(-CHEM_LDLU(lu + 26), b[24], x);
      b[79] = x;
    }
    {
      double x = b[80];
      x = fma(-CHEM_LDLU(lu + 27), b[44], x);
      b[80] = x;
    }
    {
      double x = b[81];
      b[81] = x;
    }
    {
      double x = b[82];
      x = fma(-CHEM_LDLU(lu + 28), b[44], x);
      b[82] = x;
    }
    {
      double x = b[83];
      x = fma(-CHEM_LDLU(lu + 29), b[45], x);
      b[83] = x;
    }
    {
      double x = b[84];
      x = fma(-CHEM_LDLU(lu + 30), b[71], x);
      x = fma(-CHEM_LDLU(lu + 31), b[81], x);
      b[84] = x;
    }
    {
      double x = b[85];
      b[85] = x;
    }
    {
      double x = b[86];
      x = fma(-CHEM_LDLU(lu + 32), b[41], x);
      b[86] = x;
    }
    {
      double x = b[87];
      x = fma(-CHEM_LDLU(lu + 33), b[41], x);
      x = fma(-CHEM_LDLU(lu + 34), b[51], x);
      b[87] = x;
    }
    {
      double x = b[88];
      x = fma(-CHEM_LDLU(lu + 35), b[44], x);
      b[88] = x;
    }
    {
      double x = b[89];
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
      x = fma(-CHEM_LDLU(lu + 36), b[9], x);
      x = fma(-CHEM_LDLU(lu + 37), b[10], x);
      x = fma(-CHEM_LDLU(lu + 38), b[11], x);
      b[92] = x;
    }
    {
      double x = b[93];
      b[93] = x;
    }
    {
      double x = b[94];
      x = fma(-CHEM_LDLU(lu + 39), b[70], x);
      b[94] = x;
    }
    {
      double x = b[95];
      b[95] = x;
    }
    {
      double x = b[96];
      x = fma(-CHEM_LDLU(lu + 40), b[39], x);
      x = fma(-CHEM_LDLU(lu + 41), b[86], x);
      x = fma(-CHEM_LDLU(lu + 42), b[92], x);
      b[96] = x;
    }
    {
      double x = b[97];
      x = fma(-CHEM_LDLU(lu + 43), b[10], x);
      b[97] = x;
    }
    {
      double x = b[98];
      x = fma(-CHEM_LDLU(lu + 44), b[49], x);
      b[98] = x;
    }
    {
      double x = b[99];
      x = fma(-CHEM_LDLU(lu + 45), b[98], x);
      b[99] = x;
    }
    {
      double x = b[100];
      x = fma(-CHEM_LDLU(lu + 46), b[86], x);
      x = fma(-CHEM_LDLU(lu + 47), b[98], x);
      b[100] = x;
    }
    {
      double x = b[101];
      x = fma(-CHEM_LDLU(lu + 48), b[39], x);
      x = fma(-CHEM_LDLU(lu + 49), b[86], x);
      x = fma(-CHEM_LDLU(lu + 50), b[92], x);
      x = fma(-CHEM_LDLU(lu + 51), b[98], x);
      b[101] = x;
    }
    {
      double x = b[102];
      x = fma(-CHEM_LDLU(lu + 52), b[11], x);
      b[102] = x;
    }
    {
      double x = b[103];
      x = fma(-CHEM_LDLU(lu + 53), b[9], x);
      b[103] = x;
    }
    {
      double x = b[104];
      x = fma(-CHEM_LDLU(lu + 54), b[36], x);
      b[104] = x;
    }
    {
      double x = b[105];
      x = fma(-CHEM_LDLU(lu + 55), b[38], x);
      x = fma(-CHEM_LDLU(lu + 56), b[86], x);
      x = fma(-CHEM_LDLU(lu + 57), b[98], x);
      b[105] = x;
    }
    {
      double x = b[106];
      x = fma(-CHEM_LDLU(lu + 58), b[26], x);
      b[106] = x;
    }
    {
      double x = b[107];
      x = fma(-CHEM_LDLU(lu + 59), b[27], x);
      b[107] = x;
    }
    {
      double x = b[108];
      x = fma(-CHEM_LDLU(lu + 60), b[28], x);
      b[108] = x;
    }
    {
      double x = b[109];
      x = fma(-CHEM_LDLU(lu + 61), b[31], x);
      b[109] = x;
    }
    {
      double x = b[110];
      b[110] = x;
    }
    {
      double x = b[111];
      x = fma(-CHEM_LDLU(lu + 62), b[49], x);
      x = fma(-CHEM_LDLU(lu + 63), b[98], x);
      b[111] = x;
    }
    {
      double x = b[112];
      x = fma(-CHEM_LDLU(lu + 64), b[99], x);
      x = fma(-CHEM_LDLU(lu + 65), b[105], x);
      b[112] = x;
    }
    {
      double x = b[113];
      x = fma(-CHEM_LDLU(lu + 66), b[12], x);
      x = fma(-CHEM_LDLU(lu + 67), b[13], x);
      x = fma(-CHEM_LDLU(lu + 68), b[35], x);
      x = fma(-CHEM_LDLU(lu + 69), b[39], x);
      x = fma(-CHEM_LDLU(lu + 70), b[68], x);
      x = fma(-CHEM_LDLU(lu + 71), b[86], x);
      x = fma(-CHEM_LDLU(lu + 72), b[92], x);
      x = fma(-CHEM_LDLU(lu + 73), b[98], x);
      x = fma(-CHEM_LDLU(lu + 74), b[101], x);
      b[113] = x;
    }
    {
      double x = b[114];
      x = fma(-CHEM_LDLU(lu + 75), b[39], x);
      x = fma(-CHEM_LDLU(lu + 76), b[86], x);
      x = fma(-CHEM_LDLU(lu + 77), b[92], x);
      x = fma(-CHEM_LDLU(lu + 78), b[98], x);
      x = fma(-CHEM_LDLU(lu + 79), b[101], x);
      b[114] = x;
    }
    {
      double x = b[115];
      x = fma(-CHEM_LDLU(lu + 80), b[54], x);
      x = fma(-CHEM_LDLU(lu + 81), b[112], x);
      b[115] = x;
    }
    {
      double x = b[116];
      x = fma(-CHEM_LDLU(lu + 82), b[45], x);
      b[116] = x;
    }
    {
      double x = b[117];
      x = fma(-CHEM_LDLU(lu + 83), b[44], x);
      b[117] = x;
    }
    {
      double x = b[118];
      b[118] = x;
    }
    {
      double x = b[119];
      x = fma(-CHEM_LDLU(lu + 84), b[55], x);
      x = fma(-CHEM_LDLU(lu + 85), b[86], x);
      x = fma(-CHEM_LDLU(lu + 86), b[92], x);
      x = fma(-CHEM_LDLU(lu + 87), b[95], x);
      x = fma(-CHEM_LDLU(lu + 88), b[98], x);
      x = fma(-CHEM_LDLU(lu + 89), b[101], x);
      b[119] = x;
    }
    {
      double x = b[120];
      x = fma(-CHEM_LDLU(lu + 90), b[44], x);
      b[120] = x;
    }
    {
      double x = b[121];
      x = fma(-CHEM_LDLU(lu + 91), b[49], x);
      x = fma(-CHEM_LDLU(lu + 92), b[98], x);
      b[121] = x;
    }
    {
      double x = b[122];
      x = fma(-CHEM_LDLU(lu + 93), b[25], x);
      b[122] = x;
    }
    {
      double x = b[123];
      x = fma(-CHEM_LDLU(lu + 94), b[45], x);
      b[123] = x;
    }
    {
      double x = b[124];
      b[124] = x;
    }
    {
      double x = b[125];
      x = fma(-CHEM_LDLU(lu + 95), b[36], x);
      x = fma(-CHEM_LDLU(lu + 96), b[41], x);
      x = fma(-CHEM_LDLU(lu + 97), b[44], x);
      x = fma(-CHEM_LDLU(lu + 98), b[45], x);
      x = fma(-CHEM_LDLU(lu + 99), b[86], x);
      x = fma(-CHEM_LDLU(lu + 100), b[98], x);
      b[125] = x;
    }
    {
      double x = b[126];
      x = fma(-CHEM_LDLU(lu + 101), b[36], x);
      x = fma(-CHEM_LDLU(lu + 102), b[49], x);
      x = fma(-CHEM_LDLU(lu + 103), b[70], x);
      x = fma(-CHEM_LDLU(lu + 104), b[86], x);
      x = fma(-CHEM_LDLU(lu + 105), b[98], x);
      x = fma(-CHEM_LDLU(lu + 106), b[111], x);
      b[126] = x;
    }
    {
      double x = b[127];
      x = fma(-CHEM_LDLU(lu + 107), b[36], x);
      x = fma(-CHEM_LDLU(lu + 108), b[49], x);
      x = fma(-CHEM_LDLU(lu + 109), b[70], x);
      x = fma(-CHEM_LDLU(lu + 110), b[86], x);
      x = fma(-CHEM_LDLU(lu + 111), b[98], x);
      x = fma(-CHEM_LDLU(lu + 112), b[111], x);
      x = fma(-CHEM_LDLU(lu + 113), b[126], x);
      b[127] = x;
    }
    {
      double x = b[128];
      x = fma(-CHEM_LDLU(lu + 114), b[54], x);
      x = fma(-CHEM_LDLU(lu + 115), b[80], x);
      b[128] = x;
    }
    {
      double x = b[129];
      x = fma(-CHEM_LDLU(lu + 116), b[41], x);
      x = fma(-CHEM_LDLU(lu + 117), b[42], x);
      x = fma(-CHEM_LDLU(lu + 118), b[52], x);
      b[129] = x;
    }
    {
      double x = b[130];
      x = fma(-CHEM_LDLU(lu + 119), b[44], x);
      x = fma(-CHEM_LDLU(lu + 120), b[116], x);
      x = fma(-CHEM_LDLU(lu + 121), b[117], x);
      x = fma(-CHEM_LDLU(lu + 122), b[120], x);
      x = fma(-CHEM_LDLU(lu + 123), b[123], x);
      b[130] = x;
    }
    {
      double x = b[131];
      x = fma(-CHEM_LDLU(lu + 124), b[45], x);
      x = fma(-CHEM_LDLU(lu + 125), b[116], x);
      x = fma(-CHEM_LDLU(lu + 126), b[117], x);
      x = fma(-CHEM_LDLU(lu + 127), b[120], x);
      x = fma(-CHEM_LDLU(lu + 128), b[123], x);
      x = fma(-CHEM_LDLU(lu + 129), b[130], x);
      b[131] = x;
    }
    {
      double x = b[132];
      x = fma(-CHEM_LDLU(lu + 130), b[124], x);
      b[132] = x;
    }
    {
      double x = b[133];
      x = fma(-CHEM_LDLU(lu + 131), b[54], x);
      x = fma(-CHEM_LDLU(lu + 132), b[80], x);
      x = fma(-CHEM_LDLU(lu + 133), b[116], x);
      x = fma(-CHEM_LDLU(lu + 134), b[117], x);
      x = fma(-CHEM_LDLU(lu + 135), b[120], x);
      x = fma(-CHEM_LDLU(lu + 136), b[123], x);
      x = fma(-CHEM_LDLU(lu + 137), b[130], x);
      x = fma(-CHEM_LDLU(lu + 138), b[131], x);
      b[133] = x;
    }
    {
      double x = b[134];
      x = fma(-CHEM_LDLU(lu + 139), b[41], x);
      x = fma(-CHEM_LDLU(lu + 140), b[42], x);
      x = fma(-CHEM_LDLU(lu + 141), b[116], x);
      x = fma(-CHEM_LDLU(lu + 142), b[117], x);
      x = fma(-CHEM_LDLU(lu + 143), b[120], x);
      x = fma(-CHEM_LDLU(lu + 144), b[123], x);
      x = fma(-CHEM_LDLU(lu + 145), b[130], x);
      x = fma(-CHEM_LDLU(lu + 146), b[131], x);
      b[134] = x;
    }
    {
      double x = b[135];
      x = fma(-CHEM_LDLU(lu + 147), b[97], x);
      x = fma(-CHEM_LDLU(lu + 148), b[102], x);
      x = fma(-CHEM_LDLU(lu + 149), b[105], x);
      x = fma(-CHEM_LDLU(lu + 150), b[106], x);
      x = fma(-CHEM_LDLU(lu + 151), b[107], x);
      x = fma(-CHEM_LDLU(lu + 152), b[108], x);
      b[135] = x;
    }
    {
      double x = b[136];
      x = fma(-CHEM_LDLU(lu + 153), b[8], x);
      x = fma(-CHEM_LDLU(lu + 154), b[41], x);
      x = fma(-CHEM_LDLU(lu + 155), b[44], x);
      x = fma(-CHEM_LDLU(lu + 156), b[70], x);
      x = fma(-CHEM_LDLU(lu + 157), b[86], x);
      x = fma(-CHEM_LDLU(lu + 158), b[98], x);
      x = fma(-CHEM_LDLU(lu + 159), b[111], x);
      x = fma(-CHEM_LDLU(lu + 160), b[112], x);
      x = fma(-CHEM_LDLU(lu + 161), b[121], x);
      x = fma(-CHEM_LDLU(lu + 162), b[129], x);
      x = fma(-CHEM_LDLU(lu + 163), b[134], x);
      b[136] = x;
    }
    {
      double x = b[137];
      x = fma(-CHEM_LDLU(lu + 164), b[54], x);
      x = fma(-CHEM_LDLU(lu + 165), b[80], x);
      x = fma(-CHEM_LDLU(lu + 166), b[82], x);
      x = fma(-CHEM_LDLU(lu + 167), b[83], x);
      x = fma(-CHEM_LDLU(lu + 168), b[130], x);
      x = fma(-CHEM_LDLU(lu + 169), b[131], x);
      x = fma(-CHEM_LDLU(lu + 170), b[134], x);
      b[137] = x;
    }
    {
      double x = b[138];
      x = fma(-CHEM_LDLU(lu + 171), b[63], x);
      x = fma(-CHEM_LDLU(lu + 172), b[64], x);
      x = fma(-CHEM_LDLU(lu + 173), b[65], x);
      x = fma(-CHEM_LDLU(lu + 174), b[76], x);
      x = fma(-CHEM_LDLU(lu + 175), b[77], x);
      x = fma(-CHEM_LDLU(lu + 176), b[78], x);
      x = fma(-CHEM_LDLU(lu + 177), b[79], x);
      b[138] = x;
    }
    {
      double x = b[139];
      x = fma(-CHEM_LDLU(lu + 178), b[86], x);
      x = fma(-CHEM_LDLU(lu + 179), b[97], x);
      x = fma(-CHEM_LDLU(lu + 180), b[98], x);
      x = fma(-CHEM_LDLU(lu + 181), b[102], x);
      x = fma(-CHEM_LDLU(lu + 182), b[103], x);
      x = fma(-CHEM_LDLU(lu + 183), b[105], x);
      x = fma(-CHEM_LDLU(lu + 184), b[106], x);
      x = fma(-CHEM_LDLU(lu + 185), b[109], x);
      b[139] = x;
    }
    {
      double x = b[140];
      x = fma(-CHEM_LDLU(lu + 186), b[36], x);
      x = fma(-CHEM_LDLU(lu + 187), b[86], x);
      x = fma(-CHEM_LDLU(lu + 188), b[98], x);
      x = fma(-CHEM_LDLU(lu + 189), b[100], x);
      x = fma(-CHEM_LDLU(lu + 190), b[104], x);
      x = fma(-CHEM_LDLU(lu + 191), b[130], x);
      x = fma(-CHEM_LDLU(lu + 192), b[131], x);
      x = fma(-CHEM_LDLU(lu + 193), b[134], x);
      b[140] = x;
    }
    {
      double x = b[141];
      x = fma(-CHEM_LDLU(lu + 194), b[58], x);
      x = fma(-CHEM_LDLU(lu + 195), b[97], x);
      x = fma(-CHEM_LDLU(lu + 196), b[99], x);
      x = fma(-CHEM_LDLU(lu + 197), b[102], x);
      x = fma(-CHEM_LDLU(lu + 198), b[103], x);
      x = fma(-CHEM_LDLU(lu + 199), b[105], x);
      x = fma(-CHEM_LDLU(lu + 200), b[106], x);
      x = fma(-CHEM_LDLU(lu + 201), b[107], x);
      x = fma(-CHEM_LDLU(lu + 202), b[108], x);
      b[141] = x;
    }
    {
      double x = b[142];
      x = fma(-CHEM_LDLU(lu + 203), b[44], x);
      x = fma(-CHEM_LDLU(lu + 204), b[82], x);
      x = fma(-CHEM_LDLU(lu + 205), b[116], x);
      x = fma(-CHEM_LDLU(lu + 206), b[117], x);
      x = fma(-CHEM_LDLU(lu + 207), b[120], x);
      x = fma(-CHEM_LDLU(lu + 208), b[123], x);
      x = fma(-CHEM_LDLU(lu + 209), b[130], x);
      x = fma(-CHEM_LDLU(lu + 210), b[131], x);
      x = fma(-CHEM_LDLU(lu + 211), b[134], x);
      x = fma(-CHEM_LDLU(lu + 212), b[137], x);
      b[142] = x;
    }
    {
      double x = b[143];
      x = fma(-CHEM_LDLU(lu + 213), b[45], x);
      x = fma(-CHEM_LDLU(lu + 214), b[83], x);
      x = fma(-CHEM_LDLU(lu + 215), b[116], x);
      x = fma(-CHEM_LDLU(lu + 216), b[117], x);
      x = fma(-CHEM_LDLU(lu + 217), b[120], x);
      x = fma(-CHEM_LDLU(lu + 218), b[123], x);
      x = fma(-CHEM_LDLU(lu + 219), b[130], x);
      x = fma(-CHEM_LDLU(lu + 220), b[131], x);
      x = fma(-CHEM_LDLU(lu + 221), b[134], x);
      b[143] = x;
    }
    {
      double x = b[144];
      x = fma(-CHEM_LDLU(lu + 222), b[97], x);
      x = fma(-CHEM_LDLU(lu + 223), b[102], x);
      x = fma(-CHEM_LDLU(lu + 224), b[124], x);
      x = fma(-CHEM_LDLU(lu + 225), b[132], x);
      x = fma(-CHEM_LDLU(lu + 226), b[138], x);
      b[144] = x;
    }
    {
      double x = b[145];
      x = fma(-CHEM_LDLU(lu + 227), b[106], x);
      x = fma(-CHEM_LDLU(lu + 228), b[124], x);
      x = fma(-CHEM_LDLU(lu + 229), b[132], x);
      x = fma(-CHEM_LDLU(lu + 230), b[138], x);
      b[145] = x;
    }
    {
      double x = b[146];
      x = fma(-CHEM_LDLU(lu + 231), b[41], x);
      x = fma(-CHEM_LDLU(lu + 232), b[56], x);
      x = fma(-CHEM_LDLU(lu + 233), b[57], x);
      x = fma(-CHEM_LDLU(lu + 234), b[110], x);
      x = fma(-CHEM_LDLU(lu + 235), b[111], x);
      x = fma(-CHEM_LDLU(lu + 236), b[112], x);
      x = fma(-CHEM_LDLU(lu + 237), b[129], x);
      x = fma(-CHEM_LDLU(lu + 238), b[134], x);
      b[146] = x;
    }
    {
      double x = b[147];
      x = fma(-CHEM_LDLU(lu + 239), b[63], x);
      x = fma(-CHEM_LDLU(lu + 240), b[76], x);
      x = fma(-CHEM_LDLU(lu + 241), b[77], x);
      x = fma(-CHEM_LDLU(lu + 242), b[124], x);
      x = fma(-CHEM_LDLU(lu + 243), b[132], x);
      x = fma(-CHEM_LDLU(lu + 244), b[138], x);
      x = fma(-CHEM_LDLU(lu + 245), b[145], x);
      b[147] = x;
    }
    {
      double x = b[148];
      x = fma(-CHEM_LDLU(lu + 246), b[41], x);
      x = fma(-CHEM_LDLU(lu + 247), b[42], x);
      x = fma(-CHEM_LDLU(lu + 248), b[51], x);
      x = fma(-CHEM_LDLU(lu + 249), b[52], x);
      x = fma(-CHEM_LDLU(lu + 250), b[98], x);
      x = fma(-CHEM_LDLU(lu + 251), b[116], x);
      x = fma(-CHEM_LDLU(lu + 252), b[117], x);
      x = fma(-CHEM_LDLU(lu + 253), b[120], x);
      x = fma(-CHEM_LDLU(lu + 254), b[123], x);
      x = fma(-CHEM_LDLU(lu + 255), b[130], x);
      x = fma(-CHEM_LDLU(lu + 256), b[131], x);
      x = fma(-CHEM_LDLU(lu + 257), b[134], x);
      b[148] = x;
    }
    {
      double x = b[149];
      x = fma(-CHEM_LDLU(lu + 258), b[108], x);
      x = fma(-CHEM_LDLU(lu + 259), b[138], x);
      x = fma(-CHEM_LDLU(lu + 260), b[144], x);
      x = fma(-CHEM_LDLU(lu + 261), b[145], x);
      x = fma(-CHEM_LDLU(lu + 262), b[147], x);
      b[149] = x;
    }
    {
      double x = b[150];
      x = fma(-CHEM_LDLU(lu + 263), b[44], x);
      x = fma(-CHEM_LDLU(lu + 264), b[45], x);
      x = fma(-CHEM_LDLU(lu + 265), b[48], x);
      x = fma(-CHEM_LDLU(lu + 266), b[135], x);
      x = fma(-CHEM_LDLU(lu + 267), b[142], x);
      x = fma(-CHEM_LDLU(lu + 268), b[143], x);
      b[150] = x;
    }
    {
      double x = b[151];
      x = fma(-CHEM_LDLU(lu + 269), b[50], x);
      x = fma(-CHEM_LDLU(lu + 270), b[64], x);
      x = fma(-CHEM_LDLU(lu + 271), b[65], x);
      x = fma(-CHEM_LDLU(lu + 272), b[66], x);
      x = fma(-CHEM_LDLU(lu + 273), b[77], x);
      x = fma(-CHEM_LDLU(lu + 274), b[78], x);
      x = fma(-CHEM_LDLU(lu + 275), b[79], x);
      x = fma(-CHEM_LDLU(lu + 276), b[132], x);
      x = fma(-CHEM_LDLU(lu + 277), b[138], x);
      x = fma(-CHEM_LDLU(lu + 278), b[145], x);
      x = fma(-CHEM_LDLU(lu + 279), b[147], x);
      b[151] = x;
    }
    {
      double x = b[152];
      x = fma(-CHEM_LDLU(lu + 280), b[106], x);
      x = fma(-CHEM_LDLU(lu + 281), b[107], x);
      x = fma(-CHEM_LDLU(lu + 282), b[132], x);
      x = fma(-CHEM_LDLU(lu + 283), b[138], x);
      x = fma(-CHEM_LDLU(lu + 284), b[144], x);
      x = fma(-CHEM_LDLU(lu + 285), b[145], x);
      x = fma(-CHEM_LDLU(lu + 286), b[147], x);
      x = fma(-CHEM_LDLU(lu + 287), b[151], x);
      b[152] = x;
    }
    {
      double x = b[153];
      x = fma(-CHEM_LDLU(lu + 288), b[103], x);
      x = fma(-CHEM_LDLU(lu + 289), b[105], x);
      x = fma(-CHEM_LDLU(lu + 290), b[124], x);
      x = fma(-CHEM_LDLU(lu + 291), b[132], x);
      x = fma(-CHEM_LDLU(lu + 292), b[138], x);
      x = fma(-CHEM_LDLU(lu + 293), b[144], x);
      x = fma(-CHEM_LDLU(lu + 294), b[145], x);
      x = fma(-CHEM_LDLU(lu + 295), b[147], x);
      x = fma(-CHEM_LDLU(lu + 296), b[151], x);
      x = fma(-CHEM_LDLU(lu + 297), b[152], x);
      b[153] = x;
    }
    {
      double x = b[154];
      x = fma(-CHEM_LDLU(lu + 298), b[60], x);
      x = fma(-CHEM_LDLU(lu + 299), b[97], x);
      x = fma(-CHEM_LDLU(lu + 300), b[102], x);
      x = fma(-CHEM_LDLU(lu + 301), b[124], x);
      x = fma(-CHEM_LDLU(lu + 302), b[132], x);
      x = fma(-CHEM_LDLU(lu + 303), b[138], x);
      x = fma(-CHEM_LDLU(lu + 304), b[144], x);
      x = fma(-CHEM_LDLU(lu + 305), b[145], x);
      x = fma(-CHEM_LDLU(lu + 306), b[147], x);
      x = fma(-CHEM_LDLU(lu + 307), b[151], x);
      x = fma(-CHEM_LDLU(lu + 308), b[152], x);
      x = fma(-CHEM_LDLU(lu + 309), b[153], x);
      b[154] = x;
    }
    {
      double x = b[155];
      x = fma(-CHEM_LDLU(lu + 310), b[62], x);
      x = fma(-CHEM_LDLU(lu + 311), b[63], x);
      x = fma(-CHEM_LDLU(lu + 312), b[64], x);
      x = fma(-CHEM_LDLU(lu + 313), b[72], x);
      x = fma(-CHEM_LDLU(lu + 314), b[75], x);
      x = fma(-CHEM_LDLU(lu + 315), b[76], x);
      x = fma(-CHEM_LDLU(lu + 316), b[77], x);
      x = fma(-CHEM_LDLU(lu + 317), b[78], x);
      x = fma(-CHEM_LDLU(lu + 318), b[107], x);
      x = fma(-CHEM_LDLU(lu + 319), b[132], x);
      x = fma(-CHEM_LDLU(lu + 320), b[138], x);
      x = fma(-CHEM_LDLU(lu + 321), b[145], x);
      x = fma(-CHEM_LDLU(lu + 322), b[147], x);
      x = fma(-CHEM_LDLU(lu + 323), b[151], x);
      x = fma(-CHEM_LDLU(lu + 324), b[152], x);
      x = fma(-CHEM_LDLU(lu + 325), b[153], x);
      x = fma(-CHEM_LDLU(lu + 326), b[154], x);
      b[155] = x;
    }
    {
      double x = b[156];
      x = fma(-CHEM_LDLU(lu + 327), b[61], x);
      x = fma(-CHEM_LDLU(lu + 328), b[62], x);
      x = fma(-CHEM_LDLU(lu + 329), b[72], x);
      x = fma(-CHEM_LDLU(lu + 330), b[74], x);
      x = fma(-CHEM_LDLU(lu + 331), b[75], x);
      x = fma(-CHEM_LDLU(lu + 332), b[106], x);
      x = fma(-CHEM_LDLU(lu + 333), b[107], x);
      x = fma(-CHEM_LDLU(lu + 334), b[108], x);
      x = fma(-CHEM_LDLU(lu + 335), b[124], x);
      x = fma(-CHEM_LDLU(lu + 336), b[132], x);
      x = fma(-CHEM_LDLU(lu + 337), b[138], x);
      x = fma(-CHEM_LDLU(lu + 338), b[145], x);
      x = fma(-CHEM_LDLU(lu + 339), b[147], x);
      x = fma(-CHEM_LDLU(lu + 340), b[151], x);
      x = fma(-CHEM_LDLU(lu + 341), b[152], x);
      x = fma(-CHEM_LDLU(lu + 342), b[153], x);
      x = fma(-CHEM_LDLU(lu + 343), b[154], x);
      x = fma(-CHEM_LDLU(lu + 344), b[155], x);
      b[156] = x;
    }
    {
      double x = b[157];
      x = fma(-CHEM_LDLU(lu + 345), b[3], x);
      x = fma(-CHEM_LDLU(lu + 346), b[4], x);
      x = fma(-CHEM_LDLU(lu + 347), b[32], x);
      x = fma(-CHEM_LDLU(lu + 348), b[39], x);
      x = fma(-CHEM_LDLU(lu + 349), b[55], x);
      x = fma(-CHEM_LDLU(lu + 350), b[69], x);
      x = fma(-CHEM_LDLU(lu + 351), b[86], x);
      x = fma(-CHEM_LDLU(lu + 352), b[87], x);
      x = fma(-CHEM_LDLU(lu + 353), b[92], x);
      x = fma(-CHEM_LDLU(lu + 354), b[98], x);
      x = fma(-CHEM_LDLU(lu + 355), b[101], x);
      x = fma(-CHEM_LDLU(lu + 356), b[111], x);
      x = fma(-CHEM_LDLU(lu + 357), b[129], x);
      x = fma(-CHEM_LDLU(lu + 358), b[134], x);
      x = fma(-CHEM_LDLU(lu + 359), b[139], x);
      b[157] = x;
    }
    {
      double x = b[158];
      x = fma(-CHEM_LDLU(lu + 360), b[87], x);
      x = fma(-CHEM_LDLU(lu + 361), b[89], x);
      x = fma(-CHEM_LDLU(lu + 362), b[90], x);
      x = fma(-CHEM_LDLU(lu + 363), b[91], x);
      x = fma(-CHEM_LDLU(lu + 364), b[100], x);
      x = fma(-CHEM_LDLU(lu + 365), b[104], x);
      x = fma(-CHEM_LDLU(lu + 366), b[110], x);
      x = fma(-CHEM_LDLU(lu + 367), b[111], x);
      x = fma(-CHEM_LDLU(lu + 368), b[116], x);
      x = fma(-CHEM_LDLU(lu + 369), b[117], x);
      x = fma(-CHEM_LDLU(lu + 370), b[118], x);
      x = fma(-CHEM_LDLU(lu + 371), b[120], x);
      x = fma(-CHEM_LDLU(lu + 372), b[121], x);
      x = fma(-CHEM_LDLU(lu + 373), b[123], x);
      x = fma(-CHEM_LDLU(lu + 374), b[127], x);
      x = fma(-CHEM_LDLU(lu + 375), b[129], x);
      x = fma(-CHEM_LDLU(lu + 376), b[130], x);
      x = fma(-CHEM_LDLU(lu + 377), b[131], x);
      x = fma(-CHEM_LDLU(lu + 378), b[134], x);
      x = fma(-CHEM_LDLU(lu + 379), b[137], x);
      x = fma(-CHEM_LDLU(lu + 380), b[140], x);
      x = fma(-CHEM_LDLU(lu + 381), b[142], x);
      x = fma(-CHEM_LDLU(lu + 382), b[143], x);
      x = fma(-CHEM_LDLU(lu + 383), b[146], x);
      x = fma(-CHEM_LDLU(lu + 384), b[148], x);
      x = fma(-CHEM_LDLU(lu + 385), b[152], x);
      x = fma(-CHEM_LDLU(lu + 386), b[153], x);
      x = fma(-CHEM_LDLU(lu + 387), b[154], x);
      x = fma(-CHEM_LDLU(lu + 388), b[155], x);
      x = fma(-CHEM_LDLU(lu + 389), b[156], x);
      b[158] = x;
    }
    {
      double x = b[159];
      x = fma(-CHEM_LDLU(lu + 390), b[61], x);
      x = fma(-CHEM_LDLU(lu + 391), b[62], x);
      x = fma(-CHEM_LDLU(lu + 392), b[67], x);
      x = fma(-CHEM_LDLU(lu + 393), b[74], x);
      x = fma(-CHEM_LDLU(lu + 394), b[75], x);
      x = fma(-CHEM_LDLU(lu + 395), b[76], x);
      x = fma(-CHEM_LDLU(lu + 396), b[106], x);
      x = fma(-CHEM_LDLU(lu + 397), b[108], x);
      x = fma(-CHEM_LDLU(lu + 398), b[122], x);
      x = fma(-CHEM_LDLU(lu + 399), b[124], x);
      x = fma(-CHEM_LDLU(lu + 400), b[128], x);
      x = fma(-CHEM_LDLU(lu + 401), b[130], x);
      x = fma(-CHEM_LDLU(lu + 402), b[131], x);
      x = fma(-CHEM_LDLU(lu + 403), b[132], x);
      x = fma(-CHEM_LDLU(lu + 404), b[134], x);
      x = fma(-CHEM_LDLU(lu + 405), b[138], x);
      x = fma(-CHEM_LDLU(lu + 406), b[142], x);
      x = fma(-CHEM_LDLU(lu + 407), b[143], x);
      x = fma(-CHEM_LDLU(lu + 408), b[144], x);
      x = fma(-CHEM_LDLU(lu + 409), b[145], x);
      x = fma(-CHEM_LDLU(lu + 410), b[147], x);
      x = fma(-CHEM_LDLU(lu + 411), b[151], x);
      x = fma(-CHEM_LDLU(lu + 412), b[152], x);
      x = fma(-CHEM_LDLU(lu + 413), b[153], x);
      x = fma(-CHEM_LDLU(lu + 414), b[154], x);
      x = fma(-CHEM_LDLU(lu + 415), b[155], x);
      x = fma(-CHEM_LDLU(lu + 416), b[156], x);
      b[159] = x;
    }
    {
      double x = b[160];
      x = fma(-CHEM_LDLU(lu + 417), b[35], x);
      x = fma(-CHEM_LDLU(lu + 418), b[86], x);
      x = fma(-CHEM_LDLU(lu + 419), b[98], x);
      x = fma(-CHEM_LDLU(lu + 420), b[124], x);
      x = fma(-CHEM_LDLU(lu + 421), b[132], x);
      x = fma(-CHEM_LDLU(lu + 422), b[138], x);
      x = fma(-CHEM_LDLU(lu + 423), b[145], x);
      x = fma(-CHEM_LDLU(lu + 424), b[147], x);
      x = fma(-CHEM_LDLU(lu + 425), b[151], x);
      x = fma(-CHEM_LDLU(lu + 426), b[152], x);
      x = fma(-CHEM_LDLU(lu + 427), b[153], x);
      x = fma(-CHEM_LDLU(lu + 428), b[154], x);
      x = fma(-CHEM_LDLU(lu + 429), b[155], x);
      x = fma(-CHEM_LDLU(lu + 430), b[156], x);
      x = fma(-CHEM_LDLU(lu + 431), b[159], x);
      b[160] = x;
    }
    {
      double x = b[161];
      x = fma(-CHEM_LDLU(lu + 432), b[124], x);
      x = fma(-CHEM_LDLU(lu + 433), b[132], x);
      x = fma(-CHEM_LDLU(lu + 434), b[138], x);
      x = fma(-CHEM_LDLU(lu + 435), b[144], x);
      x = fma(-CHEM_LDLU(lu + 436), b[145], x);
      x = fma(-CHEM_LDLU(lu + 437), b[147], x);
      x = fma(-CHEM_LDLU(lu + 438), b[149], x);
      x = fma(-CHEM_LDLU(lu + 439), b[151], x);
      x = fma(-CHEM_LDLU(lu + 440), b[152], x);
      x = fma(-CHEM_LDLU(lu + 441), b[153], x);
      x = fma(-CHEM_LDLU(lu + 442), b[154], x);
      x = fma(-CHEM_LDLU(lu + 443), b[155], x);
      x = fma(-CHEM_LDLU(lu + 444), b[156], x);
      x = fma(-CHEM_LDLU(lu + 445), b[159], x);
      b[161] = x;
    }
    {
      double x = b[162];
      x = fma(-CHEM_LDLU(lu + 446), b[36], x);
      x = fma(-CHEM_LDLU(lu + 447), b[41], x);
      x = fma(-CHEM_LDLU(lu + 448), b[44], x);
      x = fma(-CHEM_LDLU(lu + 449), b[45], x);
      x = fma(-CHEM_LDLU(lu + 450), b[49], x);
      x = fma(-CHEM_LDLU(lu + 451), b[50], x);
      x = fma(-CHEM_LDLU(lu + 452), b[70], x);
      x = fma(-CHEM_LDLU(lu + 453), b[73], x);
      x = fma(-CHEM_LDLU(lu + 454), b[86], x);
      x = fma(-CHEM_LDLU(lu + 455), b[98], x);
      x = fma(-CHEM_LDLU(lu + 456), b[99], x);
      x = fma(-CHEM_LDLU(lu + 457), b[111], x);
      x = fma(-CHEM_LDLU(lu + 458), b[112], x);
      x = fma(-CHEM_LDLU(lu + 459), b[119], x);
      x = fma(-CHEM_LDLU(lu + 460), b[121], x);
      x = fma(-CHEM_LDLU(lu + 461), b[129], x);
      x = fma(-CHEM_LDLU(lu + 462), b[134], x);
      x = fma(-CHEM_LDLU(lu + 463), b[135], x);
      x = fma(-CHEM_LDLU(lu + 464), b[137], x);
      x = fma(-CHEM_LDLU(lu + 465), b[139], x);
      x = fma(-CHEM_LDLU(lu + 466), b[142], x);
      x = fma(-CHEM_LDLU(lu + 467), b[143], x);
      x = fma(-CHEM_LDLU(lu + 468), b[148], x);
      b[162] = x;
    }
    {
      double x = b[163];
      x = fma(-CHEM_LDLU(lu + 469), b[34], x);
      x = fma(-CHEM_LDLU(lu + 470), b[48], x);
      x = fma(-CHEM_LDLU(lu + 471), b[90], x);
      x = fma(-CHEM_LDLU(lu + 472), b[111], x);
      x = fma(-CHEM_LDLU(lu + 473), b[115], x);
      x = fma(-CHEM_LDLU(lu + 474), b[118], x);
      x = fma(-CHEM_LDLU(lu + 475), b[121], x);
      x = fma(-CHEM_LDLU(lu + 476), b[128], x);
      x = fma(-CHEM_LDLU(lu + 477), b[129], x);
      x = fma(-CHEM_LDLU(lu + 478), b[130], x);
      x = fma(-CHEM_LDLU(lu + 479), b[131], x);
      x = fma(-CHEM_LDLU(lu + 480), b[134], x);
      x = fma(-CHEM_LDLU(lu + 481), b[135], x);
      x = fma(-CHEM_LDLU(lu + 482), b[137], x);
      x = fma(-CHEM_LDLU(lu + 483), b[142], x);
      x = fma(-CHEM_LDLU(lu + 484), b[143], x);
      x = fma(-CHEM_LDLU(lu + 485), b[144], x);
      x = fma(-CHEM_LDLU(lu + 486), b[145], x);
      x = fma(-CHEM_LDLU(lu + 487), b[147], x);
      x = fma(-CHEM_LDLU(lu + 488), b[148], x);
      x = fma(-CHEM_LDLU(lu + 489), b[150], x);
      x = fma(-CHEM_LDLU(lu + 490), b[151], x);
      x = fma(-CHEM_LDLU(lu + 491), b[152], x);
      x = fma(-CHEM_LDLU(lu + 492), b[153], x);
      x = fma(-CHEM_LDLU(lu + 493), b[154], x);
      x = fma(-CHEM_LDLU(lu + 494), b[155], x);
      x = fma(-CHEM_LDLU(lu + 495), b[156], x);
      x = fma(-CHEM_LDLU(lu + 496), b[159], x);
      x = fma(-CHEM_LDLU(lu + 497), b[160], x);
      x = fma(-CHEM_LDLU(lu + 498), b[162], x);
      b[163] = x;
    }
    {
      double x = b[164];
      x = fma(-CHEM_LDLU(lu + 499), b[41], x);
      x = fma(-CHEM_LDLU(lu + 500), b[42], x);
      x = fma(-CHEM_LDLU(lu + 501), b[90], x);
      x = fma(-CHEM_LDLU(lu + 502), b[91], x);
      x = fma(-CHEM_LDLU(lu + 503), b[97], x);
      x = fma(-CHEM_LDLU(lu + 504), b[102], x);
      x = fma(-CHEM_LDLU(lu + 505), b[103], x);
      x = fma(-CHEM_LDLU(lu + 506), b[106], x);
      x = fma(-CHEM_LDLU(lu + 507), b[107], x);
      x = fma(-CHEM_LDLU(lu + 508), b[108], x);
      x = fma(-CHEM_LDLU(lu + 509), b[111], x);
      x = fma(-CHEM_LDLU(lu + 510), b[112], x);
      x = fma(-CHEM_LDLU(lu + 511), b[118], x);
      x = fma(-CHEM_LDLU(lu + 512), b[121], x);
      x = fma(-CHEM_LDLU(lu + 513), b[129], x);
      x = fma(-CHEM_LDLU(lu + 514), b[134], x);
      x = fma(-CHEM_LDLU(lu + 515), b[135], x);
      x = fma(-CHEM_LDLU(lu + 516), b[137], x);
      x = fma(-CHEM_LDLU(lu + 517), b[142], x);
      x = fma(-CHEM_LDLU(lu + 518), b[143], x);
      x = fma(-CHEM_LDLU(lu + 519), b[148], x);
      x = fma(-CHEM_LDLU(lu + 520), b[152], x);
      x = fma(-CHEM_LDLU(lu + 521), b[153], x);
      x = fma(-CHEM_LDLU(lu + 522), b[154], x);
      x = fma(-CHEM_LDLU(lu + 523), b[155], x);
      x = fma(-CHEM_LDLU(lu + 524), b[156], x);
      x = fma(-CHEM_LDLU(lu + 525), b[159], x);
      x = fma(-CHEM_LDLU(lu + 526), b[162], x);
      b[164] = x;
    }
    {
      double x = b[165];
      x = fma(-CHEM_LDLU(lu + 527), b[86], x);
      x = fma(-CHEM_LDLU(lu + 528), b[98], x);
      x = fma(-CHEM_LDLU(lu + 529), b[100], x);
      x = fma(-CHEM_LDLU(lu + 530), b[124], x);
      x = fma(-CHEM_LDLU(lu + 531), b[132], x);
      x = fma(-CHEM_LDLU(lu + 532), b[135], x);
      x = fma(-CHEM_LDLU(lu + 533), b[138], x);
      x = fma(-CHEM_LDLU(lu + 534), b[144], x);
      x = fma(-CHEM_LDLU(lu + 535), b[145], x);
      x = fma(-CHEM_LDLU(lu + 536), b[147], x);
      x = fma(-CHEM_LDLU(lu + 537), b[149], x);
      x = fma(-CHEM_LDLU(lu + 538), b[151], x);
      x = fma(-CHEM_LDLU(lu + 539), b[152], x);
      x = fma(-CHEM_LDLU(lu + 540), b[153], x);
      x = fma(-CHEM_LDLU(lu + 541), b[154], x);
      x = fma(-CHEM_LDLU(lu + 542), b[155], x);
      x = fma(-CHEM_LDLU(lu + 543), b[156], x);
      x = fma(-CHEM_LDLU(lu + 544), b[159], x);
      x = fma(-CHEM_LDLU(lu + 545), b[160], x);
      x = fma(-CHEM_LDLU(lu + 546), b[162], x);
      b[165] = x;
    }
    {
      double x = b[166];
      x = fma(-CHEM_LDLU(lu + 547), b[26], x);
      x = fma(-CHEM_LDLU(lu + 548), b[67], x);
      x = fma(-CHEM_LDLU(lu + 549), b[74], x);
      x = fma(-CHEM_LDLU(lu + 550), b[103], x);
      x = fma(-CHEM_LDLU(lu + 551), b[105], x);
      x = fma(-CHEM_LDLU(lu + 552), b[106], x);
      x = fma(-CHEM_LDLU(lu + 553), b[107], x);
      x = fma(-CHEM_LDLU(lu + 554), b[108], x);
      x = fma(-CHEM_LDLU(lu + 555), b[122], x);
      x = fma(-CHEM_LDLU(lu + 556), b[124], x);
      x = fma(-CHEM_LDLU(lu + 557), b[128], x);
      x = fma(-CHEM_LDLU(lu + 558), b[130], x);
      x = fma(-CHEM_LDLU(lu + 559), b[131], x);
      x = fma(-CHEM_LDLU(lu + 560), b[132], x);
      x = fma(-CHEM_LDLU(lu + 561), b[134], x);
      x = fma(-CHEM_LDLU(lu + 562), b[138], x);
      x = fma(-CHEM_LDLU(lu + 563), b[142], x);
      x = fma(-CHEM_LDLU(lu + 564), b[143], x);
      x = fma(-CHEM_LDLU(lu + 565), b[144], x);
      x = fma(-CHEM_LDLU(lu + 566), b[145], x);
      x = fma(-CHEM_LDLU(lu + 567), b[147], x);
      x = fma(-CHEM_LDLU(lu + 568), b[151], x);
      x = fma(-CHEM_LDLU(lu + 569), b[152], x);
      x = fma(-CHEM_LDLU(lu + 570), b[153], x);
      x = fma(-CHEM_LDLU(lu + 571), b[154], x);
      x = fma(-CHEM_LDLU(lu + 572), b[155], x);
      x = fma(-CHEM_LDLU(lu + 573), b[156], x);
      x = fma(-CHEM_LDLU(lu + 574), b[159], x);
      x = fma(-CHEM_LDLU(lu + 575), b[162], x);
      b[166] = x;
    }
    {
      double x = b[167];
      x = fma(-CHEM_LDLU(lu + 576), b[14], x);
      x = fma(-CHEM_LDLU(lu + 577), b[36], x);
      x = fma(-CHEM_LDLU(lu + 578), b[53], x);
      x = fma(-CHEM_LDLU(lu + 579), b[57], x);
      x = fma(-CHEM_LDLU(lu + 580), b[86], x);
      x = fma(-CHEM_LDLU(lu + 581), b[98], x);
      x = fma(-CHEM_LDLU(lu + 582), b[104], x);
      x = fma(-CHEM_LDLU(lu + 583), b[110], x);
      x = fma(-CHEM_LDLU(lu + 584), b[111], x);
      x = fma(-CHEM_LDLU(lu + 585), b[114], x);
      x = fma(-CHEM_LDLU(lu + 586), b[124], x);
      x = fma(-CHEM_LDLU(lu + 587), b[129], x);
      x = fma(-CHEM_LDLU(lu + 588), b[132], x);
      x = fma(-CHEM_LDLU(lu + 589), b[134], x);
      x = fma(-CHEM_LDLU(lu + 590), b[137], x);
      x = fma(-CHEM_LDLU(lu + 591), b[138], x);
      x = fma(-CHEM_LDLU(lu + 592), b[139], x);
      x = fma(-CHEM_LDLU(lu + 593), b[142], x);
      x = fma(-CHEM_LDLU(lu + 594), b[143], x);
      x = fma(-CHEM_LDLU(lu + 595), b[145], x);
      x = fma(-CHEM_LDLU(lu + 596), b[146], x);
      x = fma(-CHEM_LDLU(lu + 597), b[147], x);
      x = fma(-CHEM_LDLU(lu + 598), b[148], x);
      x = fma(-CHEM_LDLU(lu + 599), b[151], x);
      x = fma(-CHEM_LDLU(lu + 600), b[152], x);
      x = fma(-CHEM_LDLU(lu + 601), b[153], x);
      x = fma(-CHEM_LDLU(lu + 602), b[154], x);
      x = fma(-CHEM_LDLU(lu + 603), b[155], x);
      x = fma(-CHEM_LDLU(lu + 604), b[156], x);
      x = fma(-CHEM_LDLU(lu + 605), b[159], x);
      x = fma(-CHEM_LDLU(lu + 606), b[160], x);
      x = fma(-CHEM_LDLU(lu + 607), b[162], x);
      x = fma(-CHEM_LDLU(lu + 608), b[166], x);
      b[167] = x;
    }
}
__device__ __noinline__ void solve_s1_0_1(double* __restrict__ ws, int rhs)
{
    const double* __restrict__ lu = ws + 3484;
    const double* __restrict__ vd = ws + 6769;
    double* __restrict__ b = ws + rhs;
    (void)vd;
    {
      double x = b[168];
      x = fma(-CHEM_LDLU(lu + 609), b[8], x);
      x = fma(-CHEM_LDLU(lu + 610), b[42], x);
      x = fma(-CHEM_LDLU(lu + 611), b[91], x);
      x = fma(-CHEM_LDLU(lu + 612), b[93], x);
      x = fma(-CHEM_LDLU(lu + 613), b[96], x);
      x = fma(-CHEM_LDLU(lu + 614), b[97], x);
      x = fma(-CHEM_LDLU(lu + 615), b[98], x);
      x = fma(-CHEM_LDLU(lu + 616), b[101], x);
      x = fma(-CHEM_LDLU(lu + 617), b[102], x);
      x = fma(-CHEM_LDLU(lu + 618), b[103], x);
      x = fma(-CHEM_LDLU(lu + 619), b[105], x);
      x = fma(-CHEM_LDLU(lu + 620), b[106], x);
      x = fma(-CHEM_LDLU(lu + 621), b[107], x);
      x = fma(-CHEM_LDLU(lu + 622), b[108], x);
      x = fma(-CHEM_LDLU(lu + 623), b[111], x);
      x = fma(-CHEM_LDLU(lu + 624), b[112], x);
      x = fma(-CHEM_LDLU(lu + 625), b[114], x);
      x = fma(-CHEM_LDLU(lu + 626), b[121], x);
      x = fma(-CHEM_LDLU(lu + 627), b[134], x);
      x = fma(-CHEM_LDLU(lu + 628), b[135], x);
      x = fma(-CHEM_LDLU(lu + 629), b[137], x);
      x = fma(-CHEM_LDLU(lu + 630), b[139], x);
      x = fma(-CHEM_LDLU(lu + 631), b[141], x);
      x = fma(-CHEM_LDLU(lu + 632), b[142], x);
      x = fma(-CHEM_LDLU(lu + 633), b[143], x);
      x = fma(-CHEM_LDLU(lu + 634), b[148], x);
      x = fma(-CHEM_LDLU(lu + 635), b[162], x);
      b[168] = x;
    }
    {
      double x = b[169];
      x = fma(-CHEM_LDLU(lu + 636), b[36], x);
      x = fma(-CHEM_LDLU(lu + 637), b[68], x);
      x = fma(-CHEM_LDLU(lu + 638), b[86], x);
      x = fma(-CHEM_LDLU(lu + 639), b[98], x);
      x = fma(-CHEM_LDLU(lu + 640), b[124], x);
      x = fma(-CHEM_LDLU(lu + 641), b[132], x);
      x = fma(-CHEM_LDLU(lu + 642), b[138], x);
      x = fma(-CHEM_LDLU(lu + 643), b[144], x);
      x = fma(-CHEM_LDLU(lu + 644), b[145], x);
      x = fma(-CHEM_LDLU(lu + 645), b[147], x);
      x = fma(-CHEM_LDLU(lu + 646), b[149], x);
      x = fma(-CHEM_LDLU(lu + 647), b[151], x);
      x = fma(-CHEM_LDLU(lu + 648), b[152], x);
      x = fma(-CHEM_LDLU(lu + 649), b[153], x);
      x = fma(-CHEM_LDLU(lu + 650), b[154], x);
      x = fma(-CHEM_LDLU(lu + 651), b[155], x);
      x = fma(-CHEM_LDLU(lu + 652), b[156], x);
      x = fma(-CHEM_LDLU(lu + 653), b[159], x);
      x = fma(-CHEM_LDLU(lu + 654), b[162], x);
      x = fma(-CHEM_LDLU(lu + 655), b[166], x);
      b[169] = x;
    }
    {
      double x = b[170];
      x = fma(-CHEM_LDLU(lu + 656), b[58], x);
      x = fma(-CHEM_LDLU(lu + 657), b[67], x);
      x = fma(-CHEM_LDLU(lu + 658), b[82], x);
      x = fma(-CHEM_LDLU(lu + 659), b[83], x);
      x = fma(-CHEM_LDLU(lu + 660), b[84], x);
      x = fma(-CHEM_LDLU(lu + 661), b[96], x);
      x = fma(-CHEM_LDLU(lu + 662), b[97], x);
      x = fma(-CHEM_LDLU(lu + 663), b[98], x);
      x = fma(-CHEM_LDLU(lu + 664), b[99], x);
      x = fma(-CHEM_LDLU(lu + 665), b[100], x);
      x = fma(-CHEM_LDLU(lu + 666), b[101], x);
      x = fma(-CHEM_LDLU(lu + 667), b[102], x);
      x = fma(-CHEM_LDLU(lu + 668), b[103], x);
      x = fma(-CHEM_LDLU(lu + 669), b[104], x);
      x = fma(-CHEM_LDLU(lu + 670), b[105], x);
      x = fma(-CHEM_LDLU(lu + 671), b[119], x);
      x = fma(-CHEM_LDLU(lu + 672), b[121], x);
      x = fma(-CHEM_LDLU(lu + 673), b[122], x);
      x = fma(-CHEM_LDLU(lu + 674), b[126], x);
      x = fma(-CHEM_LDLU(lu + 675), b[127], x);
      x = fma(-CHEM_LDLU(lu + 676), b[128], x);
      x = fma(-CHEM_LDLU(lu + 677), b[130], x);
      x = fma(-CHEM_LDLU(lu + 678), b[131], x);
      x = fma(-CHEM_LDLU(lu + 679), b[134], x);
      x = fma(-CHEM_LDLU(lu + 680), b[137], x);
      x = fma(-CHEM_LDLU(lu + 681), b[139], x);
      x = fma(-CHEM_LDLU(lu + 682), b[142], x);
      x = fma(-CHEM_LDLU(lu + 683), b[143], x);
      x = fma(-CHEM_LDLU(lu + 684), b[144], x);
      x = fma(-CHEM_LDLU(lu + 685), b[145], x);
      x = fma(-CHEM_LDLU(lu + 686), b[147], x);
      x = fma(-CHEM_LDLU(lu + 687), b[148], x);
      x = fma(-CHEM_LDLU(lu + 688), b[151], x);
      x = fma(-CHEM_LDLU(lu + 689), b[152], x);
      x = fma(-CHEM_LDLU(lu + 690), b[153], x);
      x = fma(-CHEM_LDLU(lu + 691), b[154], x);
      x = fma(-CHEM_LDLU(lu + 692), b[155], x);
      x = fma(-CHEM_LDLU(lu + 693), b[156], x);
      x = fma(-CHEM_LDLU(lu + 694), b[159], x);
      x = fma(-CHEM_LDLU(lu + 695), b[160], x);
      x = fma(-CHEM_LDLU(lu + 696), b[162], x);
      x = fma(-CHEM_LDLU(lu + 697), b[166], x);
      x = fma(-CHEM_LDLU(lu + 698), b[169], x);
      b[170] = x;
    }
    {
      double x = b[171];
      x = fma(-CHEM_LDLU(lu + 699), b[99], x);
      x = fma(-CHEM_LDLU(lu + 700), b[103], x);
      x = fma(-CHEM_LDLU(lu + 701), b[112], x);
      x = fma(-CHEM_LDLU(lu + 702), b[118], x);
      x = fma(-CHEM_LDLU(lu + 703), b[124], x);
      x = fma(-CHEM_LDLU(lu + 704), b[132], x);
      x = fma(-CHEM_LDLU(lu + 705), b[135], x);
      x = fma(-CHEM_LDLU(lu + 706), b[138], x);
      x = fma(-CHEM_LDLU(lu + 707), b[144], x);
      x = fma(-CHEM_LDLU(lu + 708), b[145], x);
      x = fma(-CHEM_LDLU(lu + 709), b[147], x);
      x = fma(-CHEM_LDLU(lu + 710), b[149], x);
      x = fma(-CHEM_LDLU(lu + 711), b[151], x);
      x = fma(-CHEM_LDLU(lu + 712), b[152], x);
      x = fma(-CHEM_LDLU(lu + 713), b[153], x);
      x = fma(-CHEM_LDLU(lu + 714), b[154], x);
      x = fma(-CHEM_LDLU(lu + 715), b[155], x);
      x = fma(-CHEM_LDLU(lu + 716), b[156], x);
      x = fma(-CHEM_LDLU(lu + 717), b[159], x);
      x = fma(-CHEM_LDLU(lu + 718), b[161], x);
      x = fma(-CHEM_LDLU(lu + 719), b[162], x);
      x = fma(-CHEM_LDLU(lu + 720), b[165], x);
      x = fma(-CHEM_LDLU(lu + 721), b[166], x);
      x = fma(-CHEM_LDLU(lu + 722), b[169], x);
      x = fma(-CHEM_LDLU(lu + 723), b[170], x);
      b[171] = x;
    }
    {
      double x = b[172];
      x = fma(-CHEM_LDLU(lu + 724), b[36], x);
      x = fma(-CHEM_LDLU(lu + 725), b[44], x);
      x = fma(-CHEM_LDLU(lu + 726), b[67], x);
      x = fma(-CHEM_LDLU(lu + 727), b[82], x);
      x = fma(-CHEM_LDLU(lu + 728), b[91], x);
      x = fma(-CHEM_LDLU(lu + 729), b[100], x);
      x = fma(-CHEM_LDLU(lu + 730), b[104], x);
      x = fma(-CHEM_LDLU(lu + 731), b[121], x);
      x = fma(-CHEM_LDLU(lu + 732), b[122], x);
      x = fma(-CHEM_LDLU(lu + 733), b[126], x);
      x = fma(-CHEM_LDLU(lu + 734), b[127], x);
      x = fma(-CHEM_LDLU(lu + 735), b[128], x);
      x = fma(-CHEM_LDLU(lu + 736), b[130], x);
      x = fma(-CHEM_LDLU(lu + 737), b[131], x);
      x = fma(-CHEM_LDLU(lu + 738), b[134], x);
      x = fma(-CHEM_LDLU(lu + 739), b[137], x);
      x = fma(-CHEM_LDLU(lu + 740), b[141], x);
      x = fma(-CHEM_LDLU(lu + 741), b[142], x);
      x = fma(-CHEM_LDLU(lu + 742), b[143], x);
      x = fma(-CHEM_LDLU(lu + 743), b[144], x);
      x = fma(-CHEM_LDLU(lu + 744), b[145], x);
      x = fma(-CHEM_LDLU(lu + 745), b[147], x);
      x = fma(-CHEM_LDLU(lu + 746), b[148], x);
      x = fma(-CHEM_LDLU(lu + 747), b[151], x);
      x = fma(-CHEM_LDLU(lu + 748), b[152], x);
      x = fma(-CHEM_LDLU(lu + 749), b[153], x);
      x = fma(-CHEM_LDLU(lu + 750), b[154], x);
      x = fma(-CHEM_LDLU(lu + 751), b[155], x);
      x = fma(-CHEM_LDLU(lu + 752), b[156], x);
      x = fma(-CHEM_LDLU(lu + 753), b[159], x);
      x = fma(-CHEM_LDLU(lu + 754), b[160], x);
      x = fma(-CHEM_LDLU(lu + 755), b[162], x);
      x = fma(-CHEM_LDLU(lu + 756), b[166], x);
      x = fma(-CHEM_LDLU(lu + 757), b[169], x);
      x = fma(-CHEM_LDLU(lu + 758), b[170], x);
      x = fma(-CHEM_LDLU(lu + 759), b[171], x);
      b[172] = x;
    }
    {
      double x = b[173];
      x = fma(-CHEM_LDLU(lu + 760), b[27], x);
      x = fma(-CHEM_LDLU(lu + 761), b[28], x);
      x = fma(-CHEM_LDLU(lu + 762), b[50], x);
      x = fma(-CHEM_LDLU(lu + 763), b[60], x);
      x = fma(-CHEM_LDLU(lu + 764), b[61], x);
      x = fma(-CHEM_LDLU(lu + 765), b[72], x);
      x = fma(-CHEM_LDLU(lu + 766), b[74], x);
      x = fma(-CHEM_LDLU(lu + 767), b[75], x);
      x = fma(-CHEM_LDLU(lu + 768), b[97], x);
      x = fma(-CHEM_LDLU(lu + 769), b[102], x);
      x = fma(-CHEM_LDLU(lu + 770), b[107], x);
      x = fma(-CHEM_LDLU(lu + 771), b[108], x);
      x = fma(-CHEM_LDLU(lu + 772), b[109], x);
      x = fma(-CHEM_LDLU(lu + 773), b[124], x);
      x = fma(-CHEM_LDLU(lu + 774), b[132], x);
      x = fma(-CHEM_LDLU(lu + 775), b[138], x);
      x = fma(-CHEM_LDLU(lu + 776), b[145], x);
      x = fma(-CHEM_LDLU(lu + 777), b[147], x);
      x = fma(-CHEM_LDLU(lu + 778), b[151], x);
      x = fma(-CHEM_LDLU(lu + 779), b[152], x);
      x = fma(-CHEM_LDLU(lu + 780), b[153], x);
      x = fma(-CHEM_LDLU(lu + 781), b[154], x);
      x = fma(-CHEM_LDLU(lu + 782), b[155], x);
      x = fma(-CHEM_LDLU(lu + 783), b[156], x);
      x = fma(-CHEM_LDLU(lu + 784), b[159], x);
      x = fma(-CHEM_LDLU(lu + 785), b[162], x);
      x = fma(-CHEM_LDLU(lu + 786), b[166], x);
      x = fma(-CHEM_LDLU(lu + 787), b[171], x);
      x = fma(-CHEM_LDLU(lu + 788), b[172], x);
      b[173] = x;
    }
    {
      double x = b[174];
      x = fma(-CHEM_LDLU(lu + 789), b[36], x);
      x = fma(-CHEM_LDLU(lu + 790), b[46], x);
      x = fma(-CHEM_LDLU(lu + 791), b[86], x);
      x = fma(-CHEM_LDLU(lu + 792), b[98], x);
      x = fma(-CHEM_LDLU(lu + 793), b[100], x);
      x = fma(-CHEM_LDLU(lu + 794), b[104], x);
      x = fma(-CHEM_LDLU(lu + 795), b[121], x);
      x = fma(-CHEM_LDLU(lu + 796), b[124], x);
      x = fma(-CHEM_LDLU(lu + 797), b[132], x);
      x = fma(-CHEM_LDLU(lu + 798), b[137], x);
      x = fma(-CHEM_LDLU(lu + 799), b[138], x);
      x = fma(-CHEM_LDLU(lu + 800), b[142], x);
      x = fma(-CHEM_LDLU(lu + 801), b[143], x);
      x = fma(-CHEM_LDLU(lu + 802), b[144], x);
      x = fma(-CHEM_LDLU(lu + 803), b[145], x);
      x = fma(-CHEM_LDLU(lu + 804), b[147], x);
      x = fma(-CHEM_LDLU(lu + 805), b[148], x);
      x = fma(-CHEM_LDLU(lu + 806), b[149], x);
      x = fma(-CHEM_LDLU(lu + 807), b[151], x);
      x = fma(-CHEM_LDLU(lu + 808), b[152], x);
      x = fma(-CHEM_LDLU(lu + 809), b[153], x);
      x = fma(-CHEM_LDLU(lu + 810), b[154], x);
      x = fma(-CHEM_LDLU(lu + 811), b[155], x);
      x = fma(-CHEM_LDLU(lu + 812), b[156], x);
      x = fma(-CHEM_LDLU(lu + 813), b[158], x);
      x = fma(-CHEM_LDLU(lu + 814), b[159], x);
      x = fma(-CHEM_LDLU(lu + 815), b[160], x);
      x = fma(-CHEM_LDLU(lu + 816), b[161], x);
      x = fma(-CHEM_LDLU(lu + 817), b[162], x);
      x = fma(-CHEM_LDLU(lu + 818), b[165], x);
      x = fma(-CHEM_LDLU(lu + 819), b[166], x);
      x = fma(-CHEM_LDLU(lu + 820), b[169], x);
      x = fma(-CHEM_LDLU(lu + 821), b[170], x);
      x = fma(-CHEM_LDLU(lu + 822), b[171], x);
      x = fma(-CHEM_LDLU(lu + 823), b[172], x);
      x = fma(-CHEM_LDLU(lu + 824), b[173], x);
      b[174] = x;
    }
    {
      double x = b[175];
      x = fma(-CHEM_LDLU(lu + 825), b[82], x);
      x = fma(-CHEM_LDLU(lu + 826), b[83], x);
      x = fma(-CHEM_LDLU(lu + 827), b[89], x);
      x = fma(-CHEM_LDLU(lu + 828), b[90], x);
      x = fma(-CHEM_LDLU(lu + 829), b[91], x);
      x = fma(-CHEM_LDLU(lu + 830), b[94], x);
      x = fma(-CHEM_LDLU(lu + 831), b[97], x);
      x = fma(-CHEM_LDLU(lu + 832), b[98], x);
      x = fma(-CHEM_LDLU(lu + 833), b[100], x);
      x = fma(-CHEM_LDLU(lu + 834), b[102], x);
      x = fma(-CHEM_LDLU(lu + 835), b[103], x);
      x = fma(-CHEM_LDLU(lu + 836), b[104], x);
      x = fma(-CHEM_LDLU(lu + 837), b[105], x);
      x = fma(-CHEM_LDLU(lu + 838), b[106], x);
      x = fma(-CHEM_LDLU(lu + 839), b[107], x);
      x = fma(-CHEM_LDLU(lu + 840), b[108], x);
      x = fma(-CHEM_LDLU(lu + 841), b[109], x);
      x = fma(-CHEM_LDLU(lu + 842), b[110], x);
      x = fma(-CHEM_LDLU(lu + 843), b[111], x);
      x = fma(-CHEM_LDLU(lu + 844), b[116], x);
      x = fma(-CHEM_LDLU(lu + 845), b[117], x);
      x = fma(-CHEM_LDLU(lu + 846), b[118], x);
      x = fma(-CHEM_LDLU(lu + 847), b[120], x);
      x = fma(-CHEM_LDLU(lu + 848), b[121], x);
      x = fma(-CHEM_LDLU(lu + 849), b[123], x);
      x = fma(-CHEM_LDLU(lu + 850), b[127], x);
      x = fma(-CHEM_LDLU(lu + 851), b[129], x);
      x = fma(-CHEM_LDLU(lu + 852), b[130], x);
      x = fma(-CHEM_LDLU(lu + 853), b[131], x);
      x = fma(-CHEM_LDLU(lu + 854), b[134], x);
      x = fma(-CHEM_LDLU(lu + 855), b[137], x);
      x = fma(-CHEM_LDLU(lu + 856), b[140], x);
      x = fma(-CHEM_LDLU(lu + 857), b[142], x);
      x = fma(-CHEM_LDLU(lu + 858), b[143], x);
      x = fma(-CHEM_LDLU(lu + 859), b[146], x);
      x = fma(-CHEM_LDLU(lu + 860), b[148], x);
      x = fma(-CHEM_LDLU(lu + 861), b[152], x);
      x = fma(-CHEM_LDLU(lu + 862), b[153], x);
      x = fma(-CHEM_LDLU(lu + 863), b[154], x);
      x = fma(-CHEM_LDLU(lu + 864), b[155], x);
      x = fma(-CHEM_LDLU(lu + 865), b[156], x);
      x = fma(-CHEM_LDLU(lu + 866), b[159], x);
      x = fma(-CHEM_LDLU(lu + 867), b[160], x);
      x = fma(-CHEM_LDLU(lu + 868), b[161], x);
      x = fma(-CHEM_LDLU(lu + 869), b[162], x);
      x = fma(-CHEM_LDLU(lu + 870), b[165], x);
      x = fma(-CHEM_LDLU(lu + 871), b[166], x);
      x = fma(-CHEM_LDLU(lu + 872), b[169], x);
      x = fma(-CHEM_LDLU(lu + 873), b[170], x);
      x = fma(-CHEM_LDLU(lu + 874), b[171], x);
      x = fma(-CHEM_LDLU(lu + 875), b[172], x);
      x = fma(-CHEM_LDLU(lu + 876), b[173], x);
      b[175] = x;
    }
    {
      double x = b[176];
      x = fma(-CHEM_LDLU(lu + 877), b[12], x);
      x = fma(-CHEM_LDLU(lu + 878), b[13], x);
      x = fma(-CHEM_LDLU(lu + 879), b[36], x);
      x = fma(-CHEM_LDLU(lu + 880), b[59], x);
      x = fma(-CHEM_LDLU(lu + 881), b[86], x);
      x = fma(-CHEM_LDLU(lu + 882), b[98], x);
      x = fma(-CHEM_LDLU(lu + 883), b[124], x);
      x = fma(-CHEM_LDLU(lu + 884), b[132], x);
      x = fma(-CHEM_LDLU(lu + 885), b[138], x);
      x = fma(-CHEM_LDLU(lu + 886), b[144], x);
      x = fma(-CHEM_LDLU(lu + 887), b[145], x);
      x = fma(-CHEM_LDLU(lu + 888), b[147], x);
      x = fma(-CHEM_LDLU(lu + 889), b[149], x);
      x = fma(-CHEM_LDLU(lu + 890), b[150], x);
      x = fma(-CHEM_LDLU(lu + 891), b[151], x);
      x = fma(-CHEM_LDLU(lu + 892), b[152], x);
      x = fma(-CHEM_LDLU(lu + 893), b[153], x);
      x = fma(-CHEM_LDLU(lu + 894), b[154], x);
      x = fma(-CHEM_LDLU(lu + 895), b[155], x);
      x = fma(-CHEM_LDLU(lu + 896), b[156], x);
      x = fma(-CHEM_LDLU(lu + 897), b[159], x);
      x = fma(-CHEM_LDLU(lu + 898), b[160], x);
      x = fma(-CHEM_LDLU(lu + 899), b[162], x);
      x = fma(-CHEM_LDLU(lu + 900), b[163], x);
      x = fma(-CHEM_LDLU(lu + 901), b[165], x);
      x = fma(-CHEM_LDLU(lu + 902), b[166], x);
      x = fma(-CHEM_LDLU(lu + 903), b[169], x);
      x = fma(-CHEM_LDLU(lu + 904), b[170], x);
      x = fma(-CHEM_LDLU(lu + 905), b[171], x);
      x = fma(-CHEM_LDLU(lu + 906), b[172], x);
      x = fma(-CHEM_LDLU(lu + 907), b[173], x);
      b[176] = x;
    }
    {
      double x = b[177];
      x = fma(-CHEM_LDLU(lu + 908), b[8], x);
      x = fma(-CHEM_LDLU(lu + 909), b[36], x);
      x = fma(-CHEM_LDLU(lu + 910), b[41], x);
      x = fma(-CHEM_LDLU(lu + 911), b[42], x);
      x = fma(-CHEM_LDLU(lu + 912), b[44], x);
      x = fma(-CHEM_LDLU(lu + 913), b[49], x);
      x = fma(-CHEM_LDLU(lu + 914), b[69], x);
      x = fma(-CHEM_LDLU(lu + 915), b[70], x);
      x = fma(-CHEM_LDLU(lu + 916), b[86], x);
      x = fma(-CHEM_LDLU(lu + 917), b[87], x);
      x = fma(-CHEM_LDLU(lu + 918), b[91], x);
      x = fma(-CHEM_LDLU(lu + 919), b[98], x);
      x = fma(-CHEM_LDLU(lu + 920), b[111], x);
      x = fma(-CHEM_LDLU(lu + 921), b[112], x);
      x = fma(-CHEM_LDLU(lu + 922), b[121], x);
      x = fma(-CHEM_LDLU(lu + 923), b[129], x);
      x = fma(-CHEM_LDLU(lu + 924), b[134], x);
      x = fma(-CHEM_LDLU(lu + 925), b[135], x);
      x = fma(-CHEM_LDLU(lu + 926), b[137], x);
      x = fma(-CHEM_LDLU(lu + 927), b[139], x);
      x = fma(-CHEM_LDLU(lu + 928), b[140], x);
      x = fma(-CHEM_LDLU(lu + 929), b[141], x);
      x = fma(-CHEM_LDLU(lu + 930), b[142], x);
      x = fma(-CHEM_LDLU(lu + 931), b[143], x);
      x = fma(-CHEM_LDLU(lu + 932), b[146], x);
      x = fma(-CHEM_LDLU(lu + 933), b[148], x);
      x = fma(-CHEM_LDLU(lu + 934), b[160], x);
      x = fma(-CHEM_LDLU(lu + 935), b[162], x);
      x = fma(-CHEM_LDLU(lu + 936), b[164], x);
      x = fma(-CHEM_LDLU(lu + 937), b[165], x);
      x = fma(-CHEM_LDLU(lu + 938), b[166], x);
      x = fma(-CHEM_LDLU(lu + 939), b[167], x);
      x = fma(-CHEM_LDLU(lu + 940), b[168], x);
      x = fma(-CHEM_LDLU(lu + 941), b[169], x);
      x = fma(-CHEM_LDLU(lu + 942), b[170], x);
      x = fma(-CHEM_LDLU(lu + 943), b[171], x);
      x = fma(-CHEM_LDLU(lu + 944), b[172], x);
      x = fma(-CHEM_LDLU(lu + 945), b[173], x);
      x = fma(-CHEM_LDLU(lu + 946), b[174], x);
      x = fma(-CHEM_LDLU(lu + 947), b[176], x);
      b[177] = x;
    }
    {
      double x = b[178];
      x = fma(-CHEM_LDLU(lu + 948), b[36], x);
      x = fma(-CHEM_LDLU(lu + 949), b[44], x);
      x = fma(-CHEM_LDLU(lu + 950), b[45], x);
      x = fma(-CHEM_LDLU(lu + 951), b[86], x);
      x = fma(-CHEM_LDLU(lu + 952), b[89], x);
      x = fma(-CHEM_LDLU(lu + 953), b[90], x);
      x = fma(-CHEM_LDLU(lu + 954), b[91], x);
      x = fma(-CHEM_LDLU(lu + 955), b[94], x);
      x = fma(-CHEM_LDLU(lu + 956), b[97], x);
      x = fma(-CHEM_LDLU(lu + 957), b[98], x);
      x = fma(-CHEM_LDLU(lu + 958), b[100], x);
      x = fma(-CHEM_LDLU(lu + 959), b[102], x);
      x = fma(-CHEM_LDLU(lu + 960), b[103], x);
      x = fma(-CHEM_LDLU(lu + 961), b[104], x);
      x = fma(-CHEM_LDLU(lu + 962), b[105], x);
      x = fma(-CHEM_LDLU(lu + 963), b[106], x);
      x = fma(-CHEM_LDLU(lu + 964), b[107], x);
      x = fma(-CHEM_LDLU(lu + 965), b[108], x);
      x = fma(-CHEM_LDLU(lu + 966), b[109], x);
      x = fma(-CHEM_LDLU(lu + 967), b[110], x);
      x = fma(-CHEM_LDLU(lu + 968), b[111], x);
      x = fma(-CHEM_LDLU(lu + 969), b[112], x);
      x = fma(-CHEM_LDLU(lu + 970), b[116], x);
      x = fma(-CHEM_LDLU(lu + 971), b[117], x);
      x = fma(-CHEM_LDLU(lu + 972), b[118], x);
      x = fma(-CHEM_LDLU(lu + 973), b[120], x);
      x = fma(-CHEM_LDLU(lu + 974), b[121], x);
      x = fma(-CHEM_LDLU(lu + 975), b[123], x);
      x = fma(-CHEM_LDLU(lu + 976), b[127], x);
      x = fma(-CHEM_LDLU(lu + 977), b[129], x);
      x = fma(-CHEM_LDLU(lu + 978), b[130], x);
      x = fma(-CHEM_LDLU(lu + 979), b[131], x);
      x = fma(-CHEM_LDLU(lu + 980), b[134], x);
      x = fma(-CHEM_LDLU(lu + 981), b[137], x);
      x = fma(-CHEM_LDLU(lu + 982), b[140], x);
      x = fma(-CHEM_LDLU(lu + 983), b[142], x);
      x = fma(-CHEM_LDLU(lu + 984), b[143], x);
      x = fma(-CHEM_LDLU(lu + 985), b[146], x);
      x = fma(-CHEM_LDLU(lu + 986), b[148], x);
      x = fma(-CHEM_LDLU(lu + 987), b[150], x);
      x = fma(-CHEM_LDLU(lu + 988), b[152], x);
      x = fma(-CHEM_LDLU(lu + 989), b[153], x);
      x = fma(-CHEM_LDLU(lu + 990), b[154], x);
      x = fma(-CHEM_LDLU(lu + 991), b[155], x);
      x = fma(-CHEM_LDLU(lu + 992), b[156], x);
      x = fma(-CHEM_LDLU(lu + 993), b[159], x);
      x = fma(-CHEM_LDLU(lu + 994), b[160], x);
      x = fma(-CHEM_LDLU(lu + 995), b[161], x);
      x = fma(-CHEM_LDLU(lu + 996), b[162], x);
      x = fma(-CHEM_LDLU(lu + 997), b[163], x);
      x = fma(-CHEM_LDLU(lu + 998), b[165], x);
      x = fma(-CHEM_LDLU(lu + 999), b[166], x);
      x = fma(-CHEM_LDLU(lu + 1000), b[169], x);
      x = fma(-CHEM_LDLU(lu + 1001), b[170], x);
      x = fma(-CHEM_LDLU(lu + 1002), b[171], x);
      x = fma(-CHEM_LDLU(lu + 1003), b[172], x);
      x = fma(-CHEM_LDLU(lu + 1004), b[173], x);
      x = fma(-CHEM_LDLU(lu + 1005), b[176], x);
      b[178] = x;
    }
    {
      double x = b[179];
      x = fma(-CHEM_LDLU(lu + 1006), b[58], x);
      x = fma(-CHEM_LDLU(lu + 1007), b[89], x);
      x = fma(-CHEM_LDLU(lu + 1008), b[90], x);
      x = fma(-CHEM_LDLU(lu + 1009), b[91], x);
      x = fma(-CHEM_LDLU(lu + 1010), b[93], x);
      x = fma(-CHEM_LDLU(lu + 1011), b[94], x);
      x = fma(-CHEM_LDLU(lu + 1012), b[95], x);
      x = fma(-CHEM_LDLU(lu + 1013), b[96], x);
      x = fma(-CHEM_LDLU(lu + 1014), b[97], x);
      x = fma(-CHEM_LDLU(lu + 1015), b[98], x);
      x = fma(-CHEM_LDLU(lu + 1016), b[99], x);
      x = fma(-CHEM_LDLU(lu + 1017), b[100], x);
      x = fma(-CHEM_LDLU(lu + 1018), b[101], x);
      x = fma(-CHEM_LDLU(lu + 1019), b[102], x);
      x = fma(-CHEM_LDLU(lu + 1020), b[103], x);
      x = fma(-CHEM_LDLU(lu + 1021), b[104], x);
      x = fma(-CHEM_LDLU(lu + 1022), b[105], x);
      x = fma(-CHEM_LDLU(lu + 1023), b[111], x);
      x = fma(-CHEM_LDLU(lu + 1024), b[112], x);
      x = fma(-CHEM_LDLU(lu + 1025), b[114], x);
      x = fma(-CHEM_LDLU(lu + 1026), b[118], x);
      x = fma(-CHEM_LDLU(lu + 1027), b[119], x);
      x = fma(-CHEM_LDLU(lu + 1028), b[121], x);
      x = fma(-CHEM_LDLU(lu + 1029), b[122], x);
      x = fma(-CHEM_LDLU(lu + 1030), b[124], x);
      x = fma(-CHEM_LDLU(lu + 1031), b[128], x);
      x = fma(-CHEM_LDLU(lu + 1032), b[130], x);
      x = fma(-CHEM_LDLU(lu + 1033), b[131], x);
      x = fma(-CHEM_LDLU(lu + 1034), b[132], x);
      x = fma(-CHEM_LDLU(lu + 1035), b[134], x);
      x = fma(-CHEM_LDLU(lu + 1036), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1037), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1038), b[138], x);
      x = fma(-CHEM_LDLU(lu + 1039), b[139], x);
      x = fma(-CHEM_LDLU(lu + 1040), b[140], x);
      x = fma(-CHEM_LDLU(lu + 1041), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1042), b[143], x);
      x = fma(-CHEM_LDLU(lu + 1043), b[144], x);
      x = fma(-CHEM_LDLU(lu + 1044), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1045), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1046), b[148], x);
      x = fma(-CHEM_LDLU(lu + 1047), b[151], x);
      x = fma(-CHEM_LDLU(lu + 1048), b[152], x);
      x = fma(-CHEM_LDLU(lu + 1049), b[153], x);
      x = fma(-CHEM_LDLU(lu + 1050), b[154], x);
      x = fma(-CHEM_LDLU(lu + 1051), b[155], x);
      x = fma(-CHEM_LDLU(lu + 1052), b[156], x);
      x = fma(-CHEM_LDLU(lu + 1053), b[159], x);
      x = fma(-CHEM_LDLU(lu + 1054), b[160], x);
      x = fma(-CHEM_LDLU(lu + 1055), b[161], x);
      x = fma(-CHEM_LDLU(lu + 1056), b[162], x);
      x = fma(-CHEM_LDLU(lu + 1057), b[163], x);
      x = fma(-CHEM_LDLU(lu + 1058), b[165], x);
      x = fma(-CHEM_LDLU(lu + 1059), b[166], x);
      x = fma(-CHEM_LDLU(lu + 1060), b[169], x);
      x = fma(-CHEM_LDLU(lu + 1061), b[170], x);
      x = fma(-CHEM_LDLU(lu + 1062), b[171], x);
      x = fma(-CHEM_LDLU(lu + 1063), b[172], x);
      x = fma(-CHEM_LDLU(lu + 1064), b[173], x);
      x = fma(-CHEM_LDLU(lu + 1065), b[176], x);
      x = fma(-CHEM_LDLU(lu + 1066), b[178], x);
      b[179] = x;
    }
    {
      double x = b[180];
      x = fma(-CHEM_LDLU(lu + 1067), b[14], x);
      x = fma(-CHEM_LDLU(lu + 1068), b[36], x);
      x = fma(-CHEM_LDLU(lu + 1069), b[47], x);
      x = fma(-CHEM_LDLU(lu + 1070), b[82], x);
      x = fma(-CHEM_LDLU(lu + 1071), b[86], x);
      x = fma(-CHEM_LDLU(lu + 1072), b[90], x);
      x = fma(-CHEM_LDLU(lu + 1073), b[91], x);
      x = fma(-CHEM_LDLU(lu + 1074), b[94], x);
      x = fma(-CHEM_LDLU(lu + 1075), b[98], x);
      x = fma(-CHEM_LDLU(lu + 1076), b[99], x);
      x = fma(-CHEM_LDLU(lu + 1077), b[100], x);
      x = fma(-CHEM_LDLU(lu + 1078), b[104], x);
      x = fma(-CHEM_LDLU(lu + 1079), b[111], x);
      x = fma(-CHEM_LDLU(lu + 1080), b[118], x);
      x = fma(-CHEM_LDLU(lu + 1081), b[121], x);
      x = fma(-CHEM_LDLU(lu + 1082), b[124], x);
      x = fma(-CHEM_LDLU(lu + 1083), b[126], x);
      x = fma(-CHEM_LDLU(lu + 1084), b[127], x);
      x = fma(-CHEM_LDLU(lu + 1085), b[128], x);
      x = fma(-CHEM_LDLU(lu + 1086), b[130], x);
      x = fma(-CHEM_LDLU(lu + 1087), b[131], x);
      x = fma(-CHEM_LDLU(lu + 1088), b[132], x);
      x = fma(-CHEM_LDLU(lu + 1089), b[134], x);
      x = fma(-CHEM_LDLU(lu + 1090), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1091), b[138], x);
      x = fma(-CHEM_LDLU(lu + 1092), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1093), b[143], x);
      x = fma(-CHEM_LDLU(lu + 1094), b[144], x);
      x = fma(-CHEM_LDLU(lu + 1095), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1096), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1097), b[148], x);
      x = fma(-CHEM_LDLU(lu + 1098), b[149], x);
      x = fma(-CHEM_LDLU(lu + 1099), b[151], x);
      x = fma(-CHEM_LDLU(lu + 1100), b[152], x);
      x = fma(-CHEM_LDLU(lu + 1101), b[153], x);
      x = fma(-CHEM_LDLU(lu + 1102), b[154], x);
      x = fma(-CHEM_LDLU(lu + 1103), b[155], x);
      x = fma(-CHEM_LDLU(lu + 1104), b[156], x);
      x = fma(-CHEM_LDLU(lu + 1105), b[158], x);
      x = fma(-CHEM_LDLU(lu + 1106), b[159], x);
      x = fma(-CHEM_LDLU(lu + 1107), b[160], x);
      x = fma(-CHEM_LDLU(lu + 1108), b[161], x);
      x = fma(-CHEM_LDLU(lu + 1109), b[162], x);
      x = fma(-CHEM_LDLU(lu + 1110), b[165], x);
      x = fma(-CHEM_LDLU(lu + 1111), b[166], x);
      x = fma(-CHEM_LDLU(lu + 1112), b[169], x);
      x = fma(-CHEM_LDLU(lu + 1113), b[170], x);
      x = fma(-CHEM_LDLU(lu + 1114), b[171], x);
      x = fma(-CHEM_LDLU(lu + 1115), b[172], x);
      x = fma(-CHEM_LDLU(lu + 1116), b[173], x);
      x = fma(-CHEM_LDLU(lu + 1117), b[179], x);
      b[180] = x;
    }
    {
      double x = b[181];
      x = fma(-CHEM_LDLU(lu + 1118), b[34], x);
      x = fma(-CHEM_LDLU(lu + 1119), b[36], x);
      x = fma(-CHEM_LDLU(lu + 1120), b[41], x);
      x = fma(-CHEM_LDLU(lu + 1121), b[42], x);
      x = fma(-CHEM_LDLU(lu + 1122), b[45], x);
      x = fma(-CHEM_LDLU(lu + 1123), b[71], x);
      x = fma(-CHEM_LDLU(lu + 1124), b[81], x);
      x = fma(-CHEM_LDLU(lu + 1125), b[82], x);
      x = fma(-CHEM_LDLU(lu + 1126), b[83], x);
      x = fma(-CHEM_LDLU(lu + 1127), b[89], x);
      x = fma(-CHEM_LDLU(lu + 1128), b[90], x);
      x = fma(-CHEM_LDLU(lu + 1129), b[91], x);
      x = fma(-CHEM_LDLU(lu + 1130), b[93], x);
      x = fma(-CHEM_LDLU(lu + 1131), b[94], x);
      x = fma(-CHEM_LDLU(lu + 1132), b[95], x);
      x = fma(-CHEM_LDLU(lu + 1133), b[96], x);
      x = fma(-CHEM_LDLU(lu + 1134), b[97], x);
      x = fma(-CHEM_LDLU(lu + 1135), b[98], x);
      x = fma(-CHEM_LDLU(lu + 1136), b[100], x);
      x = fma(-CHEM_LDLU(lu + 1137), b[101], x);
      x = fma(-CHEM_LDLU(lu + 1138), b[102], x);
      x = fma(-CHEM_LDLU(lu + 1139), b[103], x);
      x = fma(-CHEM_LDLU(lu + 1140), b[104], x);
      x = fma(-CHEM_LDLU(lu + 1141), b[105], x);
      x = fma(-CHEM_LDLU(lu + 1142), b[106], x);
      x = fma(-CHEM_LDLU(lu + 1143), b[107], x);
      x = fma(-CHEM_LDLU(lu + 1144), b[108], x);
      x = fma(-CHEM_LDLU(lu + 1145), b[109], x);
      x = fma(-CHEM_LDLU(lu + 1146), b[110], x);
      x = fma(-CHEM_LDLU(lu + 1147), b[111], x);
      x = fma(-CHEM_LDLU(lu + 1148), b[114], x);
      x = fma(-CHEM_LDLU(lu + 1149), b[115], x);
      x = fma(-CHEM_LDLU(lu + 1150), b[116], x);
      x = fma(-CHEM_LDLU(lu + 1151), b[117], x);
      x = fma(-CHEM_LDLU(lu + 1152), b[118], x);
      x = fma(-CHEM_LDLU(lu + 1153), b[119], x);
      x = fma(-CHEM_LDLU(lu + 1154), b[120], x);
      x = fma(-CHEM_LDLU(lu + 1155), b[121], x);
      x = fma(-CHEM_LDLU(lu + 1156), b[123], x);
      x = fma(-CHEM_LDLU(lu + 1157), b[126], x);
      x = fma(-CHEM_LDLU(lu + 1158), b[127], x);
      x = fma(-CHEM_LDLU(lu + 1159), b[129], x);
      x = fma(-CHEM_LDLU(lu + 1160), b[130], x);
      x = fma(-CHEM_LDLU(lu + 1161), b[131], x);
      x = fma(-CHEM_LDLU(lu + 1162), b[134], x);
      x = fma(-CHEM_LDLU(lu + 1163), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1164), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1165), b[139], x);
      x = fma(-CHEM_LDLU(lu + 1166), b[140], x);
      x = fma(-CHEM_LDLU(lu + 1167), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1168), b[143], x);
      x = fma(-CHEM_LDLU(lu + 1169), b[146], x);
      x = fma(-CHEM_LDLU(lu + 1170), b[148], x);
      x = fma(-CHEM_LDLU(lu + 1171), b[150], x);
      x = fma(-CHEM_LDLU(lu + 1172), b[152], x);
      x = fma(-CHEM_LDLU(lu + 1173), b[153], x);
      x = fma(-CHEM_LDLU(lu + 1174), b[154], x);
      x = fma(-CHEM_LDLU(lu + 1175), b[155], x);
      x = fma(-CHEM_LDLU(lu + 1176), b[156], x);
      x = fma(-CHEM_LDLU(lu + 1177), b[159], x);
      x = fma(-CHEM_LDLU(lu + 1178), b[160], x);
      x = fma(-CHEM_LDLU(lu + 1179), b[161], x);
      x = fma(-CHEM_LDLU(lu + 1180), b[162], x);
      x = fma(-CHEM_LDLU(lu + 1181), b[163], x);
      x = fma(-CHEM_LDLU(lu + 1182), b[164], x);
      x = fma(-CHEM_LDLU(lu + 1183), b[165], x);
      x = fma(-CHEM_LDLU(lu + 1184), b[166], x);
      x = fma(-CHEM_LDLU(lu + 1185), b[167], x);
      x = fma(-CHEM_LDLU(lu + 1186), b[169], x);
      x = fma(-CHEM_LDLU(lu + 1187), b[170], x);
      x = fma(-CHEM_LDLU(lu + 1188), b[171], x);
      x = fma(-CHEM_LDLU(lu + 1189), b[172], x);
      x = fma(-CHEM_LDLU(lu + 1190), b[173], x);
      x = fma(-CHEM_LDLU(lu + 1191), b[174], x);
      x = fma(-CHEM_LDLU(lu + 1192), b[176], x);
      x = fma(-CHEM_LDLU(lu + 1193), b[178], x);
      x = fma(-CHEM_LDLU(lu + 1194), b[179], x);
      x = fma(-CHEM_LDLU(lu + 1195), b[180], x);
      b[181] = x;
    }
    {
      double x = b[182];
      x = fma(-CHEM_LDLU(lu + 1196), b[37], x);
      x = fma(-CHEM_LDLU(lu + 1197), b[51], x);
      x = fma(-CHEM_LDLU(lu + 1198), b[54], x);
      x = fma(-CHEM_LDLU(lu + 1199), b[58], x);
      x = fma(-CHEM_LDLU(lu + 1200), b[60], x);
      x = fma(-CHEM_LDLU(lu + 1201), b[61], x);
      x = fma(-CHEM_LDLU(lu + 1202), b[62], x);
      x = fma(-CHEM_LDLU(lu + 1203), b[63], x);
      x = fma(-CHEM_LDLU(lu + 1204), b[64], x);
      x = fma(-CHEM_LDLU(lu + 1205), b[65], x);
      x = fma(-CHEM_LDLU(lu + 1206), b[66], x);
      x = fma(-CHEM_LDLU(lu + 1207), b[67], x);
      x = fma(-CHEM_LDLU(lu + 1208), b[71], x);
      x = fma(-CHEM_LDLU(lu + 1209), b[72], x);
      x = fma(-CHEM_LDLU(lu + 1210), b[73], x);
      x = fma(-CHEM_LDLU(lu + 1211), b[74], x);
      x = fma(-CHEM_LDLU(lu + 1212), b[75], x);
      x = fma(-CHEM_LDLU(lu + 1213), b[76], x);
      x = fma(-CHEM_LDLU(lu + 1214), b[77], x);
      x = fma(-CHEM_LDLU(lu + 1215), b[78], x);
      x = fma(-CHEM_LDLU(lu + 1216), b[79], x);
      x = fma(-CHEM_LDLU(lu + 1217), b[80], x);
      x = fma(-CHEM_LDLU(lu + 1218), b[81], x);
      x = fma(-CHEM_LDLU(lu + 1219), b[82], x);
      x = fma(-CHEM_LDLU(lu + 1220), b[83], x);
      x = fma(-CHEM_LDLU(lu + 1221), b[89], x);
      x = fma(-CHEM_LDLU(lu + 1222), b[90], x);
      x = fma(-CHEM_LDLU(lu + 1223), b[91], x);
      x = fma(-CHEM_LDLU(lu + 1224), b[93], x);
      x = fma(-CHEM_LDLU(lu + 1225), b[94], x);
      x = fma(-CHEM_LDLU(lu + 1226), b[95], x);
      x = fma(-CHEM_LDLU(lu + 1227), b[96], x);
      x = fma(-CHEM_LDLU(lu + 1228), b[97], x);
      x = fma(-CHEM_LDLU(lu + 1229), b[98], x);
      x = fma(-CHEM_LDLU(lu + 1230), b[99], x);
      x = fma(-CHEM_LDLU(lu + 1231), b[100], x);
      x = fma(-CHEM_LDLU(lu + 1232), b[101], x);
      x = fma(-CHEM_LDLU(lu + 1233), b[102], x);
      x = fma(-CHEM_LDLU(lu + 1234), b[103], x);
      x = fma(-CHEM_LDLU(lu + 1235), b[104], x);
      x = fma(-CHEM_LDLU(lu + 1236), b[105], x);
      x = fma(-CHEM_LDLU(lu + 1237), b[106], x);
      x = fma(-CHEM_LDLU(lu + 1238), b[107], x);
      x = fma(-CHEM_LDLU(lu + 1239), b[108], x);
      x = fma(-CHEM_LDLU(lu + 1240), b[109], x);
      x = fma(-CHEM_LDLU(lu + 1241), b[110], x);
      x = fma(-CHEM_LDLU(lu + 1242), b[111], x);
      x = fma(-CHEM_LDLU(lu + 1243), b[114], x);
      x = fma(-CHEM_LDLU(lu + 1244), b[116], x);
      x = fma(-CHEM_LDLU(lu + 1245), b[117], x);
      x = fma(-CHEM_LDLU(lu + 1246), b[118], x);
      x = fma(-CHEM_LDLU(lu + 1247), b[119], x);
      x = fma(-CHEM_LDLU(lu + 1248), b[120], x);
      x = fma(-CHEM_LDLU(lu + 1249), b[121], x);
      x = fma(-CHEM_LDLU(lu + 1250), b[122], x);
      x = fma(-CHEM_LDLU(lu + 1251), b[123], x);
      x = fma(-CHEM_LDLU(lu + 1252), b[126], x);
      x = fma(-CHEM_LDLU(lu + 1253), b[127], x);
      x = fma(-CHEM_LDLU(lu + 1254), b[128], x);
      x = fma(-CHEM_LDLU(lu + 1255), b[129], x);
      x = fma(-CHEM_LDLU(lu + 1256), b[130], x);
      x = fma(-CHEM_LDLU(lu + 1257), b[131], x);
      x = fma(-CHEM_LDLU(lu + 1258), b[134], x);
      x = fma(-CHEM_LDLU(lu + 1259), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1260), b[139], x);
      x = fma(-CHEM_LDLU(lu + 1261), b[140], x);
      x = fma(-CHEM_LDLU(lu + 1262), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1263), b[143], x);
      x = fma(-CHEM_LDLU(lu + 1264), b[144], x);
      x = fma(-CHEM_LDLU(lu + 1265), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1266), b[146], x);
      x = fma(-CHEM_LDLU(lu + 1267), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1268), b[148], x);
      x = fma(-CHEM_LDLU(lu + 1269), b[150], x);
      x = fma(-CHEM_LDLU(lu + 1270), b[151], x);
      x = fma(-CHEM_LDLU(lu + 1271), b[152], x);
      x = fma(-CHEM_LDLU(lu + 1272), b[153], x);
      x = fma(-CHEM_LDLU(lu + 1273), b[154], x);
      x = fma(-CHEM_LDLU(lu + 1274), b[155], x);
      x = fma(-CHEM_LDLU(lu + 1275), b[156], x);
      x = fma(-CHEM_LDLU(lu + 1276), b[159], x);
      x = fma(-CHEM_LDLU(lu + 1277), b[160], x);
      x = fma(-CHEM_LDLU(lu + 1278), b[161], x);
      x = fma(-CHEM_LDLU(lu + 1279), b[162], x);
      x = fma(-CHEM_LDLU(lu + 1280), b[163], x);
      x = fma(-CHEM_LDLU(lu + 1281), b[165], x);
      x = fma(-CHEM_LDLU(lu + 1282), b[166], x);
      x = fma(-CHEM_LDLU(lu + 1283), b[169], x);
      x = fma(-CHEM_LDLU(lu + 1284), b[170], x);
      x = fma(-CHEM_LDLU(lu + 1285), b[171], x);
      x = fma(-CHEM_LDLU(lu + 1286), b[172], x);
      x = fma(-CHEM_LDLU(lu + 1287), b[173], x);
      x = fma(-CHEM_LDLU(lu + 1288), b[176], x);
      x = fma(-CHEM_LDLU(lu + 1289), b[178], x);
      x = fma(-CHEM_LDLU(lu + 1290), b[179], x);
      x = fma(-CHEM_LDLU(lu + 1291), b[180], x);
      x = fma(-CHEM_LDLU(lu + 1292), b[181], x);
      b[182] = x;
    }
    {
      double x = b[183];
      x = fma(-CHEM_LDLU(lu + 1293), b[34], x);
      x = fma(-CHEM_LDLU(lu + 1294), b[36], x);
      x = fma(-CHEM_LDLU(lu + 1295), b[41], x);
      x = fma(-CHEM_LDLU(lu + 1296), b[44], x);
      x = fma(-CHEM_LDLU(lu + 1297), b[45], x);
      x = fma(-CHEM_LDLU(lu + 1298), b[48], x);
      x = fma(-CHEM_LDLU(lu + 1299), b[49], x);
      x = fma(-CHEM_LDLU(lu + 1300), b[51], x);
      x = fma(-CHEM_LDLU(lu + 1301), b[54], x);
      x = fma(-CHEM_LDLU(lu + 1302), b[69], x);
      x = fma(-CHEM_LDLU(lu + 1303), b[70], x);
      x = fma(-CHEM_LDLU(lu + 1304), b[71], x);
      x = fma(-CHEM_LDLU(lu + 1305), b[81], x);
      x = fma(-CHEM_LDLU(lu + 1306), b[82], x);
      x = fma(-CHEM_LDLU(lu + 1307), b[83], x);
      x = fma(-CHEM_LDLU(lu + 1308), b[86], x);
      x = fma(-CHEM_LDLU(lu + 1309), b[87], x);
      x = fma(-CHEM_LDLU(lu + 1310), b[88], x);
      x = fma(-CHEM_LDLU(lu + 1311), b[89], x);
      x = fma(-CHEM_LDLU(lu + 1312), b[90], x);
      x = fma(-CHEM_LDLU(lu + 1313), b[91], x);
      x = fma(-CHEM_LDLU(lu + 1314), b[93], x);
      x = fma(-CHEM_LDLU(lu + 1315), b[94], x);
      x = fma(-CHEM_LDLU(lu + 1316), b[95], x);
      x = fma(-CHEM_LDLU(lu + 1317), b[96], x);
      x = fma(-CHEM_LDLU(lu + 1318), b[97], x);
      x = fma(-CHEM_LDLU(lu + 1319), b[98], x);
      x = fma(-CHEM_LDLU(lu + 1320), b[100], x);
      x = fma(-CHEM_LDLU(lu + 1321), b[101], x);
      x = fma(-CHEM_LDLU(lu + 1322), b[102], x);
      x = fma(-CHEM_LDLU(lu + 1323), b[103], x);
      x = fma(-CHEM_LDLU(lu + 1324), b[104], x);
      x = fma(-CHEM_LDLU(lu + 1325), b[105], x);
      x = fma(-CHEM_LDLU(lu + 1326), b[106], x);
      x = fma(-CHEM_LDLU(lu + 1327), b[107], x);
      x = fma(-CHEM_LDLU(lu + 1328), b[108], x);
      x = fma(-CHEM_LDLU(lu + 1329), b[109], x);
      x = fma(-CHEM_LDLU(lu + 1330), b[110], x);
      x = fma(-CHEM_LDLU(lu + 1331), b[111], x);
      x = fma(-CHEM_LDLU(lu + 1332), b[114], x);
      x = fma(-CHEM_LDLU(lu + 1333), b[115], x);
      x = fma(-CHEM_LDLU(lu + 1334), b[116], x);
      x = fma(-CHEM_LDLU(lu + 1335), b[117], x);
      x = fma(-CHEM_LDLU(lu + 1336), b[118], x);
      x = fma(-CHEM_LDLU(lu + 1337), b[119], x);
      x = fma(-CHEM_LDLU(lu + 1338), b[120], x);
      x = fma(-CHEM_LDLU(lu + 1339), b[121], x);
      x = fma(-CHEM_LDLU(lu + 1340), b[123], x);
      x = fma(-CHEM_LDLU(lu + 1341), b[126], x);
      x = fma(-CHEM_LDLU(lu + 1342), b[127], x);
      x = fma(-CHEM_LDLU(lu + 1343), b[129], x);
      x = fma(-CHEM_LDLU(lu + 1344), b[130], x);
      x = fma(-CHEM_LDLU(lu + 1345), b[131], x);
      x = fma(-CHEM_LDLU(lu + 1346), b[134], x);
      x = fma(-CHEM_LDLU(lu + 1347), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1348), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1349), b[139], x);
      x = fma(-CHEM_LDLU(lu + 1350), b[140], x);
      x = fma(-CHEM_LDLU(lu + 1351), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1352), b[143], x);
      x = fma(-CHEM_LDLU(lu + 1353), b[146], x);
      x = fma(-CHEM_LDLU(lu + 1354), b[148], x);
      x = fma(-CHEM_LDLU(lu + 1355), b[150], x);
      x = fma(-CHEM_LDLU(lu + 1356), b[152], x);
      x = fma(-CHEM_LDLU(lu + 1357), b[153], x);
      x = fma(-CHEM_LDLU(lu + 1358), b[154], x);
      x = fma(-CHEM_LDLU(lu + 1359), b[155], x);
      x = fma(-CHEM_LDLU(lu + 1360), b[156], x);
      x = fma(-CHEM_LDLU(lu + 1361), b[159], x);
      x = fma(-CHEM_LDLU(lu + 1362), b[160], x);
      x = fma(-CHEM_LDLU(lu + 1363), b[161], x);
      x = fma(-CHEM_LDLU(lu + 1364), b[162], x);
      x = fma(-CHEM_LDLU(lu + 1365), b[163], x);
      x = fma(-CHEM_LDLU(lu + 1366), b[165], x);
      x = fma(-CHEM_LDLU(lu + 1367), b[166], x);
      x = fma(-CHEM_LDLU(lu + 1368), b[167], x);
      x = fma(-CHEM_LDLU(lu + 1369), b[168], x);
      x = fma(-CHEM_LDLU(lu + 1370), b[169], x);
      x = fma(-CHEM_LDLU(lu + 1371), b[170], x);
      x = fma(-CHEM_LDLU(lu + 1372), b[171], x);
      x = fma(-CHEM_LDLU(lu + 1373), b[172], x);
      x = fma(-CHEM_LDLU(lu + 1374), b[173], x);
      x = fma(-CHEM_LDLU(lu + 1375), b[175], x);
      x = fma(-CHEM_LDLU(lu + 1376), b[176], x);
      x = fma(-CHEM_LDLU(lu + 1377), b[178], x);
      x = fma(-CHEM_LDLU(lu + 1378), b[179], x);
      x = fma(-CHEM_LDLU(lu + 1379), b[180], x);
      x = fma(-CHEM_LDLU(lu + 1380), b[181], x);
      x = fma(-CHEM_LDLU(lu + 1381), b[182], x);
      b[183] = x;
    }
}
__device__ __noinline__ void solve_s1_0_2(double* __restrict__ ws, int rhs)
{
    const double* __restrict__ lu = ws + 3484;
    const double* __restrict__ vd = ws + 6769;
    double* __restrict__ b = ws + rhs;
    (void)vd;
    {
      double x = b[184];
      x = fma(-CHEM_LDLU(lu + 1382), b[29], x);
      x = fma(-CHEM_LDLU(lu + 1383), b[34], x);
      x = fma(-CHEM_LDLU(lu + 1384), b[36], x);
      x = fma(-CHEM_LDLU(lu + 1385), b[41], x);
      x = fma(-CHEM_LDLU(lu + 1386), b[58], x);
      x = fma(-CHEM_LDLU(lu + 1387), b[71], x);
      x = fma(-CHEM_LDLU(lu + 1388), b[81], x);
      x = fma(-CHEM_LDLU(lu + 1389), b[82], x);
      x = fma(-CHEM_LDLU(lu + 1390), b[83], x);
      x = fma(-CHEM_LDLU(lu + 1391), b[86], x);
      x = fma(-CHEM_LDLU(lu + 1392), b[88], x);
      x = fma(-CHEM_LDLU(lu + 1393), b[89], x);
      x = fma(-CHEM_LDLU(lu + 1394), b[90], x);
      x = fma(-CHEM_LDLU(lu + 1395), b[91], x);
      x = fma(-CHEM_LDLU(lu + 1396), b[93], x);
      x = fma(-CHEM_LDLU(lu + 1397), b[94], x);
      x = fma(-CHEM_LDLU(lu + 1398), b[95], x);
      x = fma(-CHEM_LDLU(lu + 1399), b[96], x);
      x = fma(-CHEM_LDLU(lu + 1400), b[97], x);
      x = fma(-CHEM_LDLU(lu + 1401), b[98], x);
      x = fma(-CHEM_LDLU(lu + 1402), b[99], x);
      x = fma(-CHEM_LDLU(lu + 1403), b[100], x);
      x = fma(-CHEM_LDLU(lu + 1404), b[101], x);
      x = fma(-CHEM_LDLU(lu + 1405), b[102], x);
      x = fma(-CHEM_LDLU(lu + 1406), b[103], x);
      x = fma(-CHEM_LDLU(lu + 1407), b[104], x);
      x = fma(-CHEM_LDLU(lu + 1408), b[105], x);
      x = fma(-CHEM_LDLU(lu + 1409), b[106], x);
      x = fma(-CHEM_LDLU(lu + 1410), b[107], x);
      x = fma(-CHEM_LDLU(lu + 1411), b[108], x);
      x = fma(-CHEM_LDLU(lu + 1412), b[109], x);
      x = fma(-CHEM_LDLU(lu + 1413), b[110], x);
      x = fma(-CHEM_LDLU(lu + 1414), b[111], x);
      x = fma(-CHEM_LDLU(lu + 1415), b[114], x);
      x = fma(-CHEM_LDLU(lu + 1416), b[115], x);
      x = fma(-CHEM_LDLU(lu + 1417), b[116], x);
      x = fma(-CHEM_LDLU(lu + 1418), b[117], x);
      x = fma(-CHEM_LDLU(lu + 1419), b[118], x);
      x = fma(-CHEM_LDLU(lu + 1420), b[119], x);
      x = fma(-CHEM_LDLU(lu + 1421), b[120], x);
      x = fma(-CHEM_LDLU(lu + 1422), b[121], x);
      x = fma(-CHEM_LDLU(lu + 1423), b[123], x);
      x = fma(-CHEM_LDLU(lu + 1424), b[124], x);
      x = fma(-CHEM_LDLU(lu + 1425), b[126], x);
      x = fma(-CHEM_LDLU(lu + 1426), b[127], x);
      x = fma(-CHEM_LDLU(lu + 1427), b[129], x);
      x = fma(-CHEM_LDLU(lu + 1428), b[130], x);
      x = fma(-CHEM_LDLU(lu + 1429), b[131], x);
      x = fma(-CHEM_LDLU(lu + 1430), b[132], x);
      x = fma(-CHEM_LDLU(lu + 1431), b[134], x);
      x = fma(-CHEM_LDLU(lu + 1432), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1433), b[138], x);
      x = fma(-CHEM_LDLU(lu + 1434), b[139], x);
      x = fma(-CHEM_LDLU(lu + 1435), b[140], x);
      x = fma(-CHEM_LDLU(lu + 1436), b[141], x);
      x = fma(-CHEM_LDLU(lu + 1437), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1438), b[143], x);
      x = fma(-CHEM_LDLU(lu + 1439), b[144], x);
      x = fma(-CHEM_LDLU(lu + 1440), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1441), b[146], x);
      x = fma(-CHEM_LDLU(lu + 1442), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1443), b[148], x);
      x = fma(-CHEM_LDLU(lu + 1444), b[149], x);
      x = fma(-CHEM_LDLU(lu + 1445), b[150], x);
      x = fma(-CHEM_LDLU(lu + 1446), b[151], x);
      x = fma(-CHEM_LDLU(lu + 1447), b[152], x);
      x = fma(-CHEM_LDLU(lu + 1448), b[153], x);
      x = fma(-CHEM_LDLU(lu + 1449), b[154], x);
      x = fma(-CHEM_LDLU(lu + 1450), b[155], x);
      x = fma(-CHEM_LDLU(lu + 1451), b[156], x);
      x = fma(-CHEM_LDLU(lu + 1452), b[159], x);
      x = fma(-CHEM_LDLU(lu + 1453), b[160], x);
      x = fma(-CHEM_LDLU(lu + 1454), b[161], x);
      x = fma(-CHEM_LDLU(lu + 1455), b[162], x);
      x = fma(-CHEM_LDLU(lu + 1456), b[163], x);
      x = fma(-CHEM_LDLU(lu + 1457), b[165], x);
      x = fma(-CHEM_LDLU(lu + 1458), b[166], x);
      x = fma(-CHEM_LDLU(lu + 1459), b[169], x);
      x = fma(-CHEM_LDLU(lu + 1460), b[170], x);
      x = fma(-CHEM_LDLU(lu + 1461), b[171], x);
      x = fma(-CHEM_LDLU(lu + 1462), b[172], x);
      x = fma(-CHEM_LDLU(lu + 1463), b[173], x);
      x = fma(-CHEM_LDLU(lu + 1464), b[174], x);
      x = fma(-CHEM_LDLU(lu + 1465), b[176], x);
      x = fma(-CHEM_LDLU(lu + 1466), b[178], x);
      x = fma(-CHEM_LDLU(lu + 1467), b[179], x);
      x = fma(-CHEM_LDLU(lu + 1468), b[180], x);
      x = fma(-CHEM_LDLU(lu + 1469), b[181], x);
      x = fma(-CHEM_LDLU(lu + 1470), b[182], x);
      b[184] = x;
    }
    {
      double x = b[185];
      x = fma(-CHEM_LDLU(lu + 1471), b[32], x);
      x = fma(-CHEM_LDLU(lu + 1472), b[34], x);
      x = fma(-CHEM_LDLU(lu + 1473), b[37], x);
      x = fma(-CHEM_LDLU(lu + 1474), b[40], x);
      x = fma(-CHEM_LDLU(lu + 1475), b[41], x);
      x = fma(-CHEM_LDLU(lu + 1476), b[48], x);
      x = fma(-CHEM_LDLU(lu + 1477), b[51], x);
      x = fma(-CHEM_LDLU(lu + 1478), b[53], x);
      x = fma(-CHEM_LDLU(lu + 1479), b[54], x);
      x = fma(-CHEM_LDLU(lu + 1480), b[57], x);
      x = fma(-CHEM_LDLU(lu + 1481), b[58], x);
      x = fma(-CHEM_LDLU(lu + 1482), b[60], x);
      x = fma(-CHEM_LDLU(lu + 1483), b[61], x);
      x = fma(-CHEM_LDLU(lu + 1484), b[62], x);
      x = fma(-CHEM_LDLU(lu + 1485), b[63], x);
      x = fma(-CHEM_LDLU(lu + 1486), b[64], x);
      x = fma(-CHEM_LDLU(lu + 1487), b[65], x);
      x = fma(-CHEM_LDLU(lu + 1488), b[66], x);
      x = fma(-CHEM_LDLU(lu + 1489), b[67], x);
      x = fma(-CHEM_LDLU(lu + 1490), b[69], x);
      x = fma(-CHEM_LDLU(lu + 1491), b[71], x);
      x = fma(-CHEM_LDLU(lu + 1492), b[72], x);
      x = fma(-CHEM_LDLU(lu + 1493), b[73], x);
      x = fma(-CHEM_LDLU(lu + 1494), b[74], x);
      x = fma(-CHEM_LDLU(lu + 1495), b[75], x);
      x = fma(-CHEM_LDLU(lu + 1496), b[76], x);
      x = fma(-CHEM_LDLU(lu + 1497), b[77], x);
      x = fma(-CHEM_LDLU(lu + 1498), b[78], x);
      x = fma(-CHEM_LDLU(lu + 1499), b[79], x);
      x = fma(-CHEM_LDLU(lu + 1500), b[80], x);
      x = fma(-CHEM_LDLU(lu + 1501), b[81], x);
      x = fma(-CHEM_LDLU(lu + 1502), b[82], x);
      x = fma(-CHEM_LDLU(lu + 1503), b[83], x);
      x = fma(-CHEM_LDLU(lu + 1504), b[84], x);
      x = fma(-CHEM_LDLU(lu + 1505), b[87], x);
      x = fma(-CHEM_LDLU(lu + 1506), b[89], x);
      x = fma(-CHEM_LDLU(lu + 1507), b[90], x);
      x = fma(-CHEM_LDLU(lu + 1508), b[91], x);
      x = fma(-CHEM_LDLU(lu + 1509), b[93], x);
      x = fma(-CHEM_LDLU(lu + 1510), b[94], x);
      x = fma(-CHEM_LDLU(lu + 1511), b[95], x);
      x = fma(-CHEM_LDLU(lu + 1512), b[96], x);
      x = fma(-CHEM_LDLU(lu + 1513), b[97], x);
      x = fma(-CHEM_LDLU(lu + 1514), b[98], x);
      x = fma(-CHEM_LDLU(lu + 1515), b[99], x);
      x = fma(-CHEM_LDLU(lu + 1516), b[100], x);
      x = fma(-CHEM_LDLU(lu + 1517), b[101], x);
      x = fma(-CHEM_LDLU(lu + 1518), b[102], x);
      x = fma(-CHEM_LDLU(lu + 1519), b[103], x);
      x = fma(-CHEM_LDLU(lu + 1520), b[104], x);
      x = fma(-CHEM_LDLU(lu + 1521), b[105], x);
      x = fma(-CHEM_LDLU(lu + 1522), b[106], x);
      x = fma(-CHEM_LDLU(lu + 1523), b[107], x);
      x = fma(-CHEM_LDLU(lu + 1524), b[108], x);
      x = fma(-CHEM_LDLU(lu + 1525), b[109], x);
      x = fma(-CHEM_LDLU(lu + 1526), b[110], x);
      x = fma(-CHEM_LDLU(lu + 1527), b[111], x);
      x = fma(-CHEM_LDLU(lu + 1528), b[114], x);
      x = fma(-CHEM_LDLU(lu + 1529), b[116], x);
      x = fma(-CHEM_LDLU(lu + 1530), b[117], x);
      x = fma(-CHEM_LDLU(lu + 1531), b[118], x);
      x = fma(-CHEM_LDLU(lu + 1532), b[119], x);
      x = fma(-CHEM_LDLU(lu + 1533), b[120], x);
      x = fma(-CHEM_LDLU(lu + 1534), b[121], x);
      x = fma(-CHEM_LDLU(lu + 1535), b[122], x);
      x = fma(-CHEM_LDLU(lu + 1536), b[123], x);
      x = fma(-CHEM_LDLU(lu + 1537), b[126], x);
      x = fma(-CHEM_LDLU(lu + 1538), b[127], x);
      x = fma(-CHEM_LDLU(lu + 1539), b[128], x);
      x = fma(-CHEM_LDLU(lu + 1540), b[129], x);
      x = fma(-CHEM_LDLU(lu + 1541), b[130], x);
      x = fma(-CHEM_LDLU(lu + 1542), b[131], x);
      x = fma(-CHEM_LDLU(lu + 1543), b[134], x);
      x = fma(-CHEM_LDLU(lu + 1544), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1545), b[139], x);
      x = fma(-CHEM_LDLU(lu + 1546), b[140], x);
      x = fma(-CHEM_LDLU(lu + 1547), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1548), b[143], x);
      x = fma(-CHEM_LDLU(lu + 1549), b[144], x);
      x = fma(-CHEM_LDLU(lu + 1550), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1551), b[146], x);
      x = fma(-CHEM_LDLU(lu + 1552), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1553), b[148], x);
      x = fma(-CHEM_LDLU(lu + 1554), b[150], x);
      x = fma(-CHEM_LDLU(lu + 1555), b[151], x);
      x = fma(-CHEM_LDLU(lu + 1556), b[152], x);
      x = fma(-CHEM_LDLU(lu + 1557), b[153], x);
      x = fma(-CHEM_LDLU(lu + 1558), b[154], x);
      x = fma(-CHEM_LDLU(lu + 1559), b[155], x);
      x = fma(-CHEM_LDLU(lu + 1560), b[156], x);
      x = fma(-CHEM_LDLU(lu + 1561), b[157], x);
      x = fma(-CHEM_LDLU(lu + 1562), b[159], x);
      x = fma(-CHEM_LDLU(lu + 1563), b[160], x);
      x = fma(-CHEM_LDLU(lu + 1564), b[161], x);
      x = fma(-CHEM_LDLU(lu + 1565), b[162], x);
      x = fma(-CHEM_LDLU(lu + 1566), b[163], x);
      x = fma(-CHEM_LDLU(lu + 1567), b[164], x);
      x = fma(-CHEM_LDLU(lu + 1568), b[165], x);
      x = fma(-CHEM_LDLU(lu + 1569), b[166], x);
      x = fma(-CHEM_LDLU(lu + 1570), b[167], x);
      x = fma(-CHEM_LDLU(lu + 1571), b[168], x);
      x = fma(-CHEM_LDLU(lu + 1572), b[169], x);
      x = fma(-CHEM_LDLU(lu + 1573), b[170], x);
      x = fma(-CHEM_LDLU(lu + 1574), b[171], x);
      x = fma(-CHEM_LDLU(lu + 1575), b[172], x);
      x = fma(-CHEM_LDLU(lu + 1576), b[173], x);
      x = fma(-CHEM_LDLU(lu + 1577), b[174], x);
      x = fma(-CHEM_LDLU(lu + 1578), b[176], x);
      x = fma(-CHEM_LDLU(lu + 1579), b[178], x);
      x = fma(-CHEM_LDLU(lu + 1580), b[179], x);
      x = fma(-CHEM_LDLU(lu + 1581), b[180], x);
      x = fma(-CHEM_LDLU(lu + 1582), b[181], x);
      x = fma(-CHEM_LDLU(lu + 1583), b[182], x);
      x = fma(-CHEM_LDLU(lu + 1584), b[183], x);
      x = fma(-CHEM_LDLU(lu + 1585), b[184], x);
      b[185] = x;
    }
    {
      double x = b[186];
      x = fma(-CHEM_LDLU(lu + 1586), b[32], x);
      x = fma(-CHEM_LDLU(lu + 1587), b[34], x);
      x = fma(-CHEM_LDLU(lu + 1588), b[36], x);
      x = fma(-CHEM_LDLU(lu + 1589), b[39], x);
      x = fma(-CHEM_LDLU(lu + 1590), b[40], x);
      x = fma(-CHEM_LDLU(lu + 1591), b[41], x);
      x = fma(-CHEM_LDLU(lu + 1592), b[44], x);
      x = fma(-CHEM_LDLU(lu + 1593), b[45], x);
      x = fma(-CHEM_LDLU(lu + 1594), b[48], x);
      x = fma(-CHEM_LDLU(lu + 1595), b[49], x);
      x = fma(-CHEM_LDLU(lu + 1596), b[50], x);
      x = fma(-CHEM_LDLU(lu + 1597), b[53], x);
      x = fma(-CHEM_LDLU(lu + 1598), b[55], x);
      x = fma(-CHEM_LDLU(lu + 1599), b[57], x);
      x = fma(-CHEM_LDLU(lu + 1600), b[60], x);
      x = fma(-CHEM_LDLU(lu + 1601), b[61], x);
      x = fma(-CHEM_LDLU(lu + 1602), b[62], x);
      x = fma(-CHEM_LDLU(lu + 1603), b[63], x);
      x = fma(-CHEM_LDLU(lu + 1604), b[64], x);
      x = fma(-CHEM_LDLU(lu + 1605), b[65], x);
      x = fma(-CHEM_LDLU(lu + 1606), b[66], x);
      x = fma(-CHEM_LDLU(lu + 1607), b[67], x);
      x = fma(-CHEM_LDLU(lu + 1608), b[70], x);
      x = fma(-CHEM_LDLU(lu + 1609), b[71], x);
      x = fma(-CHEM_LDLU(lu + 1610), b[72], x);
      x = fma(-CHEM_LDLU(lu + 1611), b[73], x);
      x = fma(-CHEM_LDLU(lu + 1612), b[74], x);
      x = fma(-CHEM_LDLU(lu + 1613), b[75], x);
      x = fma(-CHEM_LDLU(lu + 1614), b[76], x);
      x = fma(-CHEM_LDLU(lu + 1615), b[77], x);
      x = fma(-CHEM_LDLU(lu + 1616), b[78], x);
      x = fma(-CHEM_LDLU(lu + 1617), b[79], x);
      x = fma(-CHEM_LDLU(lu + 1618), b[81], x);
      x = fma(-CHEM_LDLU(lu + 1619), b[82], x);
      x = fma(-CHEM_LDLU(lu + 1620), b[83], x);
      x = fma(-CHEM_LDLU(lu + 1621), b[86], x);
      x = fma(-CHEM_LDLU(lu + 1622), b[89], x);
      x = fma(-CHEM_LDLU(lu + 1623), b[90], x);
      x = fma(-CHEM_LDLU(lu + 1624), b[91], x);
      x = fma(-CHEM_LDLU(lu + 1625), b[92], x);
      x = fma(-CHEM_LDLU(lu + 1626), b[93], x);
      x = fma(-CHEM_LDLU(lu + 1627), b[94], x);
      x = fma(-CHEM_LDLU(lu + 1628), b[95], x);
      x = fma(-CHEM_LDLU(lu + 1629), b[96], x);
      x = fma(-CHEM_LDLU(lu + 1630), b[97], x);
      x = fma(-CHEM_LDLU(lu + 1631), b[98], x);
      x = fma(-CHEM_LDLU(lu + 1632), b[99], x);
      x = fma(-CHEM_LDLU(lu + 1633), b[100], x);
      x = fma(-CHEM_LDLU(lu + 1634), b[101], x);
      x = fma(-CHEM_LDLU(lu + 1635), b[102], x);
      x = fma(-CHEM_LDLU(lu + 1636), b[103], x);
      x = fma(-CHEM_LDLU(lu + 1637), b[104], x);
      x = fma(-CHEM_LDLU(lu + 1638), b[105], x);
      x = fma(-CHEM_LDLU(lu + 1639), b[106], x);
      x = fma(-CHEM_LDLU(lu + 1640), b[107], x);
      x = fma(-CHEM_LDLU(lu + 1641), b[108], x);
      x = fma(-CHEM_LDLU(lu + 1642), b[109], x);
      x = fma(-CHEM_LDLU(lu + 1643), b[110], x);
      x = fma(-CHEM_LDLU(lu + 1644), b[111], x);
      x = fma(-CHEM_LDLU(lu + 1645), b[114], x);
      x = fma(-CHEM_LDLU(lu + 1646), b[118], x);
      x = fma(-CHEM_LDLU(lu + 1647), b[119], x);
      x = fma(-CHEM_LDLU(lu + 1648), b[121], x);
      x = fma(-CHEM_LDLU(lu + 1649), b[122], x);
      x = fma(-CHEM_LDLU(lu + 1650), b[126], x);
      x = fma(-CHEM_LDLU(lu + 1651), b[127], x);
      x = fma(-CHEM_LDLU(lu + 1652), b[128], x);
      x = fma(-CHEM_LDLU(lu + 1653), b[129], x);
      x = fma(-CHEM_LDLU(lu + 1654), b[130], x);
      x = fma(-CHEM_LDLU(lu + 1655), b[131], x);
      x = fma(-CHEM_LDLU(lu + 1656), b[134], x);
      x = fma(-CHEM_LDLU(lu + 1657), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1658), b[139], x);
      x = fma(-CHEM_LDLU(lu + 1659), b[140], x);
      x = fma(-CHEM_LDLU(lu + 1660), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1661), b[143], x);
      x = fma(-CHEM_LDLU(lu + 1662), b[144], x);
      x = fma(-CHEM_LDLU(lu + 1663), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1664), b[146], x);
      x = fma(-CHEM_LDLU(lu + 1665), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1666), b[148], x);
      x = fma(-CHEM_LDLU(lu + 1667), b[150], x);
      x = fma(-CHEM_LDLU(lu + 1668), b[151], x);
      x = fma(-CHEM_LDLU(lu + 1669), b[152], x);
      x = fma(-CHEM_LDLU(lu + 1670), b[153], x);
      x = fma(-CHEM_LDLU(lu + 1671), b[154], x);
      x = fma(-CHEM_LDLU(lu + 1672), b[155], x);
      x = fma(-CHEM_LDLU(lu + 1673), b[156], x);
      x = fma(-CHEM_LDLU(lu + 1674), b[157], x);
      x = fma(-CHEM_LDLU(lu + 1675), b[159], x);
      x = fma(-CHEM_LDLU(lu + 1676), b[160], x);
      x = fma(-CHEM_LDLU(lu + 1677), b[161], x);
      x = fma(-CHEM_LDLU(lu + 1678), b[162], x);
      x = fma(-CHEM_LDLU(lu + 1679), b[163], x);
      x = fma(-CHEM_LDLU(lu + 1680), b[164], x);
      x = fma(-CHEM_LDLU(lu + 1681), b[165], x);
      x = fma(-CHEM_LDLU(lu + 1682), b[166], x);
      x = fma(-CHEM_LDLU(lu + 1683), b[167], x);
      x = fma(-CHEM_LDLU(lu + 1684), b[168], x);
      x = fma(-CHEM_LDLU(lu + 1685), b[169], x);
      x = fma(-CHEM_LDLU(lu + 1686), b[170], x);
      x = fma(-CHEM_LDLU(lu + 1687), b[171], x);
      x = fma(-CHEM_LDLU(lu + 1688), b[172], x);
      x = fma(-CHEM_LDLU(lu + 1689), b[173], x);
      x = fma(-CHEM_LDLU(lu + 1690), b[174], x);
      x = fma(-CHEM_LDLU(lu + 1691), b[176], x);
      x = fma(-CHEM_LDLU(lu + 1692), b[178], x);
      x = fma(-CHEM_LDLU(lu + 1693), b[179], x);
      x = fma(-CHEM_LDLU(lu + 1694), b[180], x);
      x = fma(-CHEM_LDLU(lu + 1695), b[181], x);
      x = fma(-CHEM_LDLU(lu + 1696), b[182], x);
      x = fma(-CHEM_LDLU(lu + 1697), b[183], x);
      x = fma(-CHEM_LDLU(lu + 1698), b[184], x);
      x = fma(-CHEM_LDLU(lu + 1699), b[185], x);
      b[186] = x;
    }
    {
      double x = b[187];
      x = fma(-CHEM_LDLU(lu + 1700), b[5], x);
      x = fma(-CHEM_LDLU(lu + 1701), b[8], x);
      x = fma(-CHEM_LDLU(lu + 1702), b[9], x);
      x = fma(-CHEM_LDLU(lu + 1703), b[10], x);
      x = fma(-CHEM_LDLU(lu + 1704), b[11], x);
      x = fma(-CHEM_LDLU(lu + 1705), b[14], x);
      x = fma(-CHEM_LDLU(lu + 1706), b[26], x);
      x = fma(-CHEM_LDLU(lu + 1707), b[27], x);
      x = fma(-CHEM_LDLU(lu + 1708), b[28], x);
      x = fma(-CHEM_LDLU(lu + 1709), b[36], x);
      x = fma(-CHEM_LDLU(lu + 1710), b[38], x);
      x = fma(-CHEM_LDLU(lu + 1711), b[39], x);
      x = fma(-CHEM_LDLU(lu + 1712), b[40], x);
      x = fma(-CHEM_LDLU(lu + 1713), b[41], x);
      x = fma(-CHEM_LDLU(lu + 1714), b[42], x);
      x = fma(-CHEM_LDLU(lu + 1715), b[44], x);
      x = fma(-CHEM_LDLU(lu + 1716), b[46], x);
      x = fma(-CHEM_LDLU(lu + 1717), b[47], x);
      x = fma(-CHEM_LDLU(lu + 1718), b[49], x);
      x = fma(-CHEM_LDLU(lu + 1719), b[51], x);
      x = fma(-CHEM_LDLU(lu + 1720), b[54], x);
      x = fma(-CHEM_LDLU(lu + 1721), b[58], x);
      x = fma(-CHEM_LDLU(lu + 1722), b[60], x);
      x = fma(-CHEM_LDLU(lu + 1723), b[61], x);
      x = fma(-CHEM_LDLU(lu + 1724), b[62], x);
      x = fma(-CHEM_LDLU(lu + 1725), b[63], x);
      x = fma(-CHEM_LDLU(lu + 1726), b[64], x);
      x = fma(-CHEM_LDLU(lu + 1727), b[65], x);
      x = fma(-CHEM_LDLU(lu + 1728), b[66], x);
      x = fma(-CHEM_LDLU(lu + 1729), b[67], x);
      x = fma(-CHEM_LDLU(lu + 1730), b[69], x);
      x = fma(-CHEM_LDLU(lu + 1731), b[70], x);
      x = fma(-CHEM_LDLU(lu + 1732), b[71], x);
      x = fma(-CHEM_LDLU(lu + 1733), b[72], x);
      x = fma(-CHEM_LDLU(lu + 1734), b[74], x);
      x = fma(-CHEM_LDLU(lu + 1735), b[75], x);
      x = fma(-CHEM_LDLU(lu + 1736), b[76], x);
      x = fma(-CHEM_LDLU(lu + 1737), b[77], x);
      x = fma(-CHEM_LDLU(lu + 1738), b[78], x);
      x = fma(-CHEM_LDLU(lu + 1739), b[79], x);
      x = fma(-CHEM_LDLU(lu + 1740), b[80], x);
      x = fma(-CHEM_LDLU(lu + 1741), b[81], x);
      x = fma(-CHEM_LDLU(lu + 1742), b[82], x);
      x = fma(-CHEM_LDLU(lu + 1743), b[83], x);
      x = fma(-CHEM_LDLU(lu + 1744), b[86], x);
      x = fma(-CHEM_LDLU(lu + 1745), b[87], x);
      x = fma(-CHEM_LDLU(lu + 1746), b[88], x);
      x = fma(-CHEM_LDLU(lu + 1747), b[89], x);
      x = fma(-CHEM_LDLU(lu + 1748), b[90], x);
      x = fma(-CHEM_LDLU(lu + 1749), b[91], x);
      x = fma(-CHEM_LDLU(lu + 1750), b[92], x);
      x = fma(-CHEM_LDLU(lu + 1751), b[93], x);
      x = fma(-CHEM_LDLU(lu + 1752), b[94], x);
      x = fma(-CHEM_LDLU(lu + 1753), b[95], x);
      x = fma(-CHEM_LDLU(lu + 1754), b[96], x);
      x = fma(-CHEM_LDLU(lu + 1755), b[97], x);
      x = fma(-CHEM_LDLU(lu + 1756), b[98], x);
      x = fma(-CHEM_LDLU(lu + 1757), b[99], x);
      x = fma(-CHEM_LDLU(lu + 1758), b[100], x);
      x = fma(-CHEM_LDLU(lu + 1759), b[101], x);
      x = fma(-CHEM_LDLU(lu + 1760), b[102], x);
      x = fma(-CHEM_LDLU(lu + 1761), b[103], x);
      x = fma(-CHEM_LDLU(lu + 1762), b[104], x);
      x = fma(-CHEM_LDLU(lu + 1763), b[105], x);
      x = fma(-CHEM_LDLU(lu + 1764), b[106], x);
      x = fma(-CHEM_LDLU(lu + 1765), b[107], x);
      x = fma(-CHEM_LDLU(lu + 1766), b[108], x);
      x = fma(-CHEM_LDLU(lu + 1767), b[109], x);
      x = fma(-CHEM_LDLU(lu + 1768), b[110], x);
      x = fma(-CHEM_LDLU(lu + 1769), b[111], x);
      x = fma(-CHEM_LDLU(lu + 1770), b[112], x);
      x = fma(-CHEM_LDLU(lu + 1771), b[114], x);
      x = fma(-CHEM_LDLU(lu + 1772), b[116], x);
      x = fma(-CHEM_LDLU(lu + 1773), b[117], x);
      x = fma(-CHEM_LDLU(lu + 1774), b[118], x);
      x = fma(-CHEM_LDLU(lu + 1775), b[119], x);
      x = fma(-CHEM_LDLU(lu + 1776), b[120], x);
      x = fma(-CHEM_LDLU(lu + 1777), b[121], x);
      x = fma(-CHEM_LDLU(lu + 1778), b[122], x);
      x = fma(-CHEM_LDLU(lu + 1779), b[123], x);
      x = fma(-CHEM_LDLU(lu + 1780), b[125], x);
      x = fma(-CHEM_LDLU(lu + 1781), b[126], x);
      x = fma(-CHEM_LDLU(lu + 1782), b[127], x);
      x = fma(-CHEM_LDLU(lu + 1783), b[128], x);
      x = fma(-CHEM_LDLU(lu + 1784), b[129], x);
      x = fma(-CHEM_LDLU(lu + 1785), b[130], x);
      x = fma(-CHEM_LDLU(lu + 1786), b[131], x);
      x = fma(-CHEM_LDLU(lu + 1787), b[134], x);
      x = fma(-CHEM_LDLU(lu + 1788), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1789), b[136], x);
      x = fma(-CHEM_LDLU(lu + 1790), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1791), b[139], x);
      x = fma(-CHEM_LDLU(lu + 1792), b[140], x);
      x = fma(-CHEM_LDLU(lu + 1793), b[141], x);
      x = fma(-CHEM_LDLU(lu + 1794), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1795), b[143], x);
      x = fma(-CHEM_LDLU(lu + 1796), b[144], x);
      x = fma(-CHEM_LDLU(lu + 1797), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1798), b[146], x);
      x = fma(-CHEM_LDLU(lu + 1799), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1800), b[148], x);
      x = fma(-CHEM_LDLU(lu + 1801), b[150], x);
      x = fma(-CHEM_LDLU(lu + 1802), b[151], x);
      x = fma(-CHEM_LDLU(lu + 1803), b[152], x);
      x = fma(-CHEM_LDLU(lu + 1804), b[153], x);
      x = fma(-CHEM_LDLU(lu + 1805), b[154], x);
      x = fma(-CHEM_LDLU(lu + 1806), b[155], x);
      x = fma(-CHEM_LDLU(lu + 1807), b[156], x);
      x = fma(-CHEM_LDLU(lu + 1808), b[158], x);
      x = fma(-CHEM_LDLU(lu + 1809), b[159], x);
      x = fma(-CHEM_LDLU(lu + 1810), b[160], x);
      x = fma(-CHEM_LDLU(lu + 1811), b[161], x);
      x = fma(-CHEM_LDLU(lu + 1812), b[162], x);
      x = fma(-CHEM_LDLU(lu + 1813), b[163], x);
      x = fma(-CHEM_LDLU(lu + 1814), b[164], x);
      x = fma(-CHEM_LDLU(lu + 1815), b[165], x);
      x = fma(-CHEM_LDLU(lu + 1816), b[166], x);
      x = fma(-CHEM_LDLU(lu + 1817), b[167], x);
      x = fma(-CHEM_LDLU(lu + 1818), b[168], x);
      x = fma(-CHEM_LDLU(lu + 1819), b[169], x);
      x = fma(-CHEM_LDLU(lu + 1820), b[170], x);
      x = fma(-CHEM_LDLU(lu + 1821), b[171], x);
      x = fma(-CHEM_LDLU(lu + 1822), b[172], x);
      x = fma(-CHEM_LDLU(lu + 1823), b[173], x);
      x = fma(-CHEM_LDLU(lu + 1824), b[174], x);
      x = fma(-CHEM_LDLU(lu + 1825), b[175], x);
      x = fma(-CHEM_LDLU(lu + 1826), b[176], x);
      x = fma(-CHEM_LDLU(lu + 1827), b[177], x);
      x = fma(-CHEM_LDLU(lu + 1828), b[178], x);
      x = fma(-CHEM_LDLU(lu + 1829), b[179], x);
      x = fma(-CHEM_LDLU(lu + 1830), b[180], x);
      x = fma(-CHEM_LDLU(lu + 1831), b[181], x);
      x = fma(-CHEM_LDLU(lu + 1832), b[182], x);
      x = fma(-CHEM_LDLU(lu + 1833), b[183], x);
      x = fma(-CHEM_LDLU(lu + 1834), b[184], x);
      x = fma(-CHEM_LDLU(lu + 1835), b[185], x);
      x = fma(-CHEM_LDLU(lu + 1836), b[186], x);
      b[187] = x;
    }
    {
      double x = b[188];
      x = fma(-CHEM_LDLU(lu + 1837), b[5], x);
      x = fma(-CHEM_LDLU(lu + 1838), b[8], x);
      x = fma(-CHEM_LDLU(lu + 1839), b[9], x);
      x = fma(-CHEM_LDLU(lu + 1840), b[10], x);
      x = fma(-CHEM_LDLU(lu + 1841), b[11], x);
      x = fma(-CHEM_LDLU(lu + 1842), b[12], x);
      x = fma(-CHEM_LDLU(lu + 1843), b[13], x);
      x = fma(-CHEM_LDLU(lu + 1844), b[14], x);
      x = fma(-CHEM_LDLU(lu + 1845), b[18], x);
      x = fma(-CHEM_LDLU(lu + 1846), b[19], x);
      x = fma(-CHEM_LDLU(lu + 1847), b[20], x);
      x = fma(-CHEM_LDLU(lu + 1848), b[21], x);
      x = fma(-CHEM_LDLU(lu + 1849), b[22], x);
      x = fma(-CHEM_LDLU(lu + 1850), b[23], x);
      x = fma(-CHEM_LDLU(lu + 1851), b[24], x);
      x = fma(-CHEM_LDLU(lu + 1852), b[25], x);
      x = fma(-CHEM_LDLU(lu + 1853), b[26], x);
      x = fma(-CHEM_LDLU(lu + 1854), b[27], x);
      x = fma(-CHEM_LDLU(lu + 1855), b[28], x);
      x = fma(-CHEM_LDLU(lu + 1856), b[29], x);
      x = fma(-CHEM_LDLU(lu + 1857), b[31], x);
      x = fma(-CHEM_LDLU(lu + 1858), b[34], x);
      x = fma(-CHEM_LDLU(lu + 1859), b[35], x);
      x = fma(-CHEM_LDLU(lu + 1860), b[36], x);
      x = fma(-CHEM_LDLU(lu + 1861), b[37], x);
      x = fma(-CHEM_LDLU(lu + 1862), b[38], x);
      x = fma(-CHEM_LDLU(lu + 1863), b[39], x);
      x = fma(-CHEM_LDLU(lu + 1864), b[40], x);
      x = fma(-CHEM_LDLU(lu + 1865), b[41], x);
      x = fma(-CHEM_LDLU(lu + 1866), b[42], x);
      x = fma(-CHEM_LDLU(lu + 1867), b[43], x);
      x = fma(-CHEM_LDLU(lu + 1868), b[44], x);
      x = fma(-CHEM_LDLU(lu + 1869), b[45], x);
      x = fma(-CHEM_LDLU(lu + 1870), b[46], x);
      x = fma(-CHEM_LDLU(lu + 1871), b[47], x);
      x = fma(-CHEM_LDLU(lu + 1872), b[48], x);
      x = fma(-CHEM_LDLU(lu + 1873), b[49], x);
      x = fma(-CHEM_LDLU(lu + 1874), b[50], x);
      x = fma(-CHEM_LDLU(lu + 1875), b[51], x);
      x = fma(-CHEM_LDLU(lu + 1876), b[52], x);
      x = fma(-CHEM_LDLU(lu + 1877), b[53], x);
      x = fma(-CHEM_LDLU(lu + 1878), b[54], x);
      x = fma(-CHEM_LDLU(lu + 1879), b[55], x);
      x = fma(-CHEM_LDLU(lu + 1880), b[56], x);
      x = fma(-CHEM_LDLU(lu + 1881), b[57], x);
      x = fma(-CHEM_LDLU(lu + 1882), b[58], x);
      x = fma(-CHEM_LDLU(lu + 1883), b[59], x);
      x = fma(-CHEM_LDLU(lu + 1884), b[68], x);
      x = fma(-CHEM_LDLU(lu + 1885), b[69], x);
      x = fma(-CHEM_LDLU(lu + 1886), b[70], x);
      x = fma(-CHEM_LDLU(lu + 1887), b[80], x);
      x = fma(-CHEM_LDLU(lu + 1888), b[82], x);
      x = fma(-CHEM_LDLU(lu + 1889), b[83], x);
      x = fma(-CHEM_LDLU(lu + 1890), b[86], x);
      x = fma(-CHEM_LDLU(lu + 1891), b[87], x);
      x = fma(-CHEM_LDLU(lu + 1892), b[88], x);
      x = fma(-CHEM_LDLU(lu + 1893), b[89], x);
      x = fma(-CHEM_LDLU(lu + 1894), b[92], x);
      x = fma(-CHEM_LDLU(lu + 1895), b[94], x);
      x = fma(-CHEM_LDLU(lu + 1896), b[98], x);
      x = fma(-CHEM_LDLU(lu + 1897), b[99], x);
      x = fma(-CHEM_LDLU(lu + 1898), b[101], x);
      x = fma(-CHEM_LDLU(lu + 1899), b[110], x);
      x = fma(-CHEM_LDLU(lu + 1900), b[111], x);
      x = fma(-CHEM_LDLU(lu + 1901), b[112], x);
      x = fma(-CHEM_LDLU(lu + 1902), b[115], x);
      x = fma(-CHEM_LDLU(lu + 1903), b[116], x);
      x = fma(-CHEM_LDLU(lu + 1904), b[117], x);
      x = fma(-CHEM_LDLU(lu + 1905), b[120], x);
      x = fma(-CHEM_LDLU(lu + 1906), b[121], x);
      x = fma(-CHEM_LDLU(lu + 1907), b[123], x);
      x = fma(-CHEM_LDLU(lu + 1908), b[124], x);
      x = fma(-CHEM_LDLU(lu + 1909), b[125], x);
      x = fma(-CHEM_LDLU(lu + 1910), b[128], x);
      x = fma(-CHEM_LDLU(lu + 1911), b[129], x);
      x = fma(-CHEM_LDLU(lu + 1912), b[130], x);
      x = fma(-CHEM_LDLU(lu + 1913), b[131], x);
      x = fma(-CHEM_LDLU(lu + 1914), b[132], x);
      x = fma(-CHEM_LDLU(lu + 1915), b[134], x);
      x = fma(-CHEM_LDLU(lu + 1916), b[135], x);
      x = fma(-CHEM_LDLU(lu + 1917), b[136], x);
      x = fma(-CHEM_LDLU(lu + 1918), b[137], x);
      x = fma(-CHEM_LDLU(lu + 1919), b[138], x);
      x = fma(-CHEM_LDLU(lu + 1920), b[139], x);
      x = fma(-CHEM_LDLU(lu + 1921), b[140], x);
      x = fma(-CHEM_LDLU(lu + 1922), b[141], x);
      x = fma(-CHEM_LDLU(lu + 1923), b[142], x);
      x = fma(-CHEM_LDLU(lu + 1924), b[143], x);
      x = fma(-CHEM_LDLU(lu + 1925), b[144], x);
      x = fma(-CHEM_LDLU(lu + 1926), b[145], x);
      x = fma(-CHEM_LDLU(lu + 1927), b[146], x);
      x = fma(-CHEM_LDLU(lu + 1928), b[147], x);
      x = fma(-CHEM_LDLU(lu + 1929), b[148], x);
      x = fma(-CHEM_LDLU(lu + 1930), b[149], x);
      x = fma(-CHEM_LDLU(lu + 1931), b[150], x);
      x = fma(-CHEM_LDLU(lu + 1932), b[151], x);
      x = fma(-CHEM_LDLU(lu + 1933), b[152], x);
      x = fma(-CHEM_LDLU(lu + 1934), b[153], x);
      x = fma(-CHEM_LDLU(lu + 1935), b[154], x);
      x = fma(-CHEM_LDLU(lu + 1936), b[155], x);
      x = fma(-CHEM_LDLU(lu + 1937), b[156], x);
      x = fma(-CHEM_LDLU(lu + 1938), b[157], x);
      x = fma(-CHEM_LDLU(lu + 1939), b[158], x);
      x = fma(-CHEM_LDLU(lu + 1940), b[159], x);
      x = fma(-CHEM_LDLU(lu + 1941), b[160], x);
      x = fma(-CHEM_LDLU(lu + 1942), b[161], x);
      x = fma(-CHEM_LDLU(lu + 1943), b[162], x);
      x = fma(-CHEM_LDLU(lu + 1944), b[163], x);
      x = fma(-CHEM_LDLU(lu + 1945), b[164], x);
      x = fma(-CHEM_LDLU(lu + 1946), b[165], x);
      x = fma(-CHEM_LDLU(lu + 1947), b[166], x);
      x = fma(-CHEM_LDLU(lu + 1948), b[167], x);
      x = fma(-CHEM_LDLU(lu + 1949), b[168], x);
      x = fma(-CHEM_LDLU(lu + 1950), b[169], x);
      x = fma(-CHEM_LDLU(lu + 1951), b[170], x);
      x = fma(-CHEM_LDLU(lu + 1952), b[171], x);
      x = fma(-CHEM_LDLU(lu + 1953), b[172], x);
      x = fma(-CHEM_LDLU(lu + 1954), b[173], x);
      x = fma(-CHEM_LDLU(lu + 1955), b[174], x);
      x = fma(-CHEM_LDLU(lu + 1956), b[175], x);
      x = fma(-CHEM_LDLU(lu + 1957), b[176], x);
      x = fma(-CHEM_LDLU(lu + 1958), b[177], x);
      x = fma(-CHEM_LDLU(lu + 1959), b[178], x);
      x = fma(-CHEM_LDLU(lu + 1960), b[179], x);
      x = fma(-CHEM_LDLU(lu + 1961), b[180], x);
      x = fma(-CHEM_LDLU(lu + 1962), b[181], x);
      x = fma(-CHEM_LDLU(lu + 1963), b[182], x);
      x = fma(-CHEM_LDLU(lu + 1964), b[183], x);
      x = fma(-CHEM_LDLU(lu + 1965), b[184], x);
      x = fma(-CHEM_LDLU(lu + 1966), b[185], x);
      x = fma(-CHEM_LDLU(lu + 1967), b[186], x);
      x = fma(-CHEM_LDLU(lu + 1968), b[187], x);
      b[188] = x;
    }
    {
      double x = b[188];
      b[188] = x * CHEM_LDLU(vd + 188);
    }
    {
      double x = b[187];
      x = fma(-CHEM_LDLU(lu + 1969), b[188], x);
      b[187] = x * CHEM_LDLU(vd + 187);
    }
    {
      double x = b[186];
      x = fma(-CHEM_LDLU(lu + 1970), b[187], x);
      x = fma(-CHEM_LDLU(lu + 1971), b[188], x);
      b[186] = x * CHEM_LDLU(vd + 186);
    }
    {
      double x = b[185];
      x = fma(-CHEM_LDLU(lu + 1972), b[186], x);
      x = fma(-CHEM_LDLU(lu + 1973), b[187], x);
      x = fma(-CHEM_LDLU(lu + 1974), b[188], x);
      b[185] = x * CHEM_LDLU(vd + 185);
    }
    {
      double x = b[184];
      x = fma(-CHEM_LDLU(lu + 1975), b[185], x);
      x = fma(-CHEM_LDLU(lu + 1976), b[186], x);
      x = fma(-CHEM_LDLU(lu + 1977), b[187], x);
      x = fma(-CHEM_LDLU(lu + 1978), b[188], x);
      b[184] = x * CHEM_LDLU(vd + 184);
    }
    {
      double x = b[183];
      x = fma(-CHEM_LDLU(lu + 1979), b[184], x);
      x = fma(-CHEM_LDLU(lu + 1980), b[185], x);
      x = fma(-CHEM_LDLU(lu + 1981), b[186], x);
      x = fma(-CHEM_LDLU(lu + 1982), b[187], x);
      x = fma(-CHEM_LDLU(lu + 1983), b[188], x);
      b[183] = x * CHEM_LDLU(vd + 183);
    }
    {
      double x = b[182];
      x = fma(-CHEM_LDLU(lu + 1984), b[184], x);
      x = fma(-CHEM_LDLU(lu + 1985), b[185], x);
      x = fma(-CHEM_LDLU(lu + 1986), b[186], x);
      x = fma(-CHEM_LDLU(lu + 1987), b[187], x);
      x = fma(-CHEM_LDLU(lu + 1988), b[188], x);
      b[182] = x * CHEM_LDLU(vd + 182);
    }
    {
      double x = b[181];
      x = fma(-CHEM_LDLU(lu + 1989), b[182], x);
      x = fma(-CHEM_LDLU(lu + 1990), b[184], x);
      x = fma(-CHEM_LDLU(lu + 1991), b[185], x);
      x = fma(-CHEM_LDLU(lu + 1992), b[186], x);
      x = fma(-CHEM_LDLU(lu + 1993), b[187], x);
      x = fma(-CHEM_LDLU(lu + 1994), b[188], x);
      b[181] = x * CHEM_LDLU(vd + 181);
    }
    {
      double x = b[180];
      x = fma(-CHEM_LDLU(lu + 1995), b[181], x);
      x = fma(-CHEM_LDLU(lu + 1996), b[182], x);
      x = fma(-CHEM_LDLU(lu + 1997), b[184], x);
      x = fma(-CHEM_LDLU(lu + 1998), b[185], x);
      x = fma(-CHEM_LDLU(lu + 1999), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2000), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2001), b[188], x);
      b[180] = x * CHEM_LDLU(vd + 180);
    }
    {
      double x = b[179];
      x = fma(-CHEM_LDLU(lu + 2002), b[180], x);
      x = fma(-CHEM_LDLU(lu + 2003), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2004), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2005), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2006), b[185], x);
      x = fma(-CHEM_LDLU(lu + 2007), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2008), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2009), b[188], x);
      b[179] = x * CHEM_LDLU(vd + 179);
    }
    {
      double x = b[178];
      x = fma(-CHEM_LDLU(lu + 2010), b[179], x);
      x = fma(-CHEM_LDLU(lu + 2011), b[180], x);
      x = fma(-CHEM_LDLU(lu + 2012), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2013), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2014), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2015), b[185], x);
      x = fma(-CHEM_LDLU(lu + 2016), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2017), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2018), b[188], x);
      b[178] = x * CHEM_LDLU(vd + 178);
    }
    {
      double x = b[177];
      x = fma(-CHEM_LDLU(lu + 2019), b[178], x);
      x = fma(-CHEM_LDLU(lu + 2020), b[179], x);
      x = fma(-CHEM_LDLU(lu + 2021), b[180], x);
      x = fma(-CHEM_LDLU(lu + 2022), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2023), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2024), b[183], x);
      x = fma(-CHEM_LDLU(lu + 2025), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2026), b[185], x);
      x = fma(-CHEM_LDLU(lu + 2027), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2028), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2029), b[188], x);
      b[177] = x * CHEM_LDLU(vd + 177);
    }
    {
      double x = b[176];
      x = fma(-CHEM_LDLU(lu + 2030), b[179], x);
      x = fma(-CHEM_LDLU(lu + 2031), b[180], x);
      x = fma(-CHEM_LDLU(lu + 2032), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2033), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2034), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2035), b[185], x);
      x = fma(-CHEM_LDLU(lu + 2036), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2037), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2038), b[188], x);
      b[176] = x * CHEM_LDLU(vd + 176);
    }
    {
      double x = b[175];
      x = fma(-CHEM_LDLU(lu + 2039), b[176], x);
      x = fma(-CHEM_LDLU(lu + 2040), b[179], x);
      x = fma(-CHEM_LDLU(lu + 2041), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2042), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2043), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2044), b[185], x);
      x = fma(-CHEM_LDLU(lu + 2045), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2046), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2047), b[188], x);
      b[175] = x * CHEM_LDLU(vd + 175);
    }
    {
      double x = b[174];
      x = fma(-CHEM_LDLU(lu + 2048), b[176], x);
      x = fma(-CHEM_LDLU(lu + 2049), b[179], x);
      x = fma(-CHEM_LDLU(lu + 2050), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2051), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2052), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2053), b[185], x);
      x = fma(-CHEM_LDLU(lu + 2054), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2055), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2056), b[188], x);
      b[174] = x * CHEM_LDLU(vd + 174);
    }
    {
      double x = b[173];
      x = fma(-CHEM_LDLU(lu + 2057), b[179], x);
      x = fma(-CHEM_LDLU(lu + 2058), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2059), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2060), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2061), b[185], x);
      x = fma(-CHEM_LDLU(lu + 2062), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2063), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2064), b[188], x);
      b[173] = x * CHEM_LDLU(vd + 173);
    }
    {
      double x = b[172];
      x = fma(-CHEM_LDLU(lu + 2065), b[173], x);
      x = fma(-CHEM_LDLU(lu + 2066), b[179], x);
      x = fma(-CHEM_LDLU(lu + 2067), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2068), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2069), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2070), b[185], x);
      x = fma(-CHEM_LDLU(lu + 2071), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2072), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2073), b[188], x);
      b[172] = x * CHEM_LDLU(vd + 172);
    }
    {
      double x = b[171];
      x = fma(-CHEM_LDLU(lu + 2074), b[172], x);
      x = fma(-CHEM_LDLU(lu + 2075), b[173], x);
      x = fma(-CHEM_LDLU(lu + 2076), b[179], x);
      x = fma(-CHEM_LDLU(lu + 2077), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2078), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2079), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2080), b[185], x);
      x = fma(-CHEM_LDLU(lu + 2081), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2082), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2083), b[188], x);
      b[171] = x * CHEM_LDLU(vd + 171);
    }
    {
      double x = b[170];
      x = fma(-CHEM_LDLU(lu + 2084), b[171], x);
      x = fma(-CHEM_LDLU(lu + 2085), b[173], x);
      x = fma(-CHEM_LDLU(lu + 2086), b[179], x);
      x = fma(-CHEM_LDLU(lu + 2087), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2088), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2089), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2090), b[185], x);
      x = fma(-CHEM_LDLU(lu + 2091), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2092), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2093), b[188], x);
      b[170] = x * CHEM_LDLU(vd + 170);
    }
    {
      double x = b[169];
      x = fma(-CHEM_LDLU(lu + 2094), b[170], x);
      x = fma(-CHEM_LDLU(lu + 2095), b[171], x);
      x = fma(-CHEM_LDLU(lu + 2096), b[173], x);
      x = fma(-CHEM_LDLU(lu + 2097), b[179], x);
      x = fma(-CHEM_LDLU(lu + 2098), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2099), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2100), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2101), b[185], x);
      x = fma(-CHEM_LDLU(lu + 2102), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2103), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2104), b[188], x);
      b[169] = x * CHEM_LDLU(vd + 169);
    }
    {
      double x = b[168];
      x = fma(-CHEM_LDLU(lu + 2105), b[169], x);
      x = fma(-CHEM_LDLU(lu + 2106), b[171], x);
      x = fma(-CHEM_LDLU(lu + 2107), b[178], x);
      x = fma(-CHEM_LDLU(lu + 2108), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2109), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2110), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2111), b[185], x);
      x = fma(-CHEM_LDLU(lu + 2112), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2113), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2114), b[188], x);
      b[168] = x * CHEM_LDLU(vd + 168);
    }
    {
      double x = b[167];
      x = fma(-CHEM_LDLU(lu + 2115), b[171], x);
      x = fma(-CHEM_LDLU(lu + 2116), b[173], x);
      x = fma(-CHEM_LDLU(lu + 2117), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2118), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2119), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2120), b[185], x);
      x = fma(-CHEM_LDLU(lu + 2121), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2122), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2123), b[188], x);
      b[167] = x * CHEM_LDLU(vd + 167);
    }
    {
      double x = b[166];
      x = fma(-CHEM_LDLU(lu + 2124), b[171], x);
      x = fma(-CHEM_LDLU(lu + 2125), b[173], x);
      x = fma(-CHEM_LDLU(lu + 2126), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2127), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2128), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2129), b[185], x);
      x = fma(-CHEM_LDLU(lu + 2130), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2131), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2132), b[188], x);
      b[166] = x * CHEM_LDLU(vd + 166);
    }
    {
      double x = b[165];
      x = fma(-CHEM_LDLU(lu + 2133), b[166], x);
      x = fma(-CHEM_LDLU(lu + 2134), b[169], x);
      x = fma(-CHEM_LDLU(lu + 2135), b[171], x);
      x = fma(-CHEM_LDLU(lu + 2136), b[173], x);
      x = fma(-CHEM_LDLU(lu + 2137), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2138), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2139), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2140), b[185], x);
      x = fma(-CHEM_LDLU(lu + 2141), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2142), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2143), b[188], x);
      b[165] = x * CHEM_LDLU(vd + 165);
    }
}
__device__ __noinline__ void solve_s1_0_3(double* __restrict__ ws, int rhs)
{
    const double* __restrict__ lu = ws + 3484;
    const double* __restrict__ vd = ws + 6769;
    double* __restrict__ b = ws + rhs;
    (void)vd;
    {
      double x = b[164];
      x = fma(-CHEM_LDLU(lu + 2144), b[166], x);
      x = fma(-CHEM_LDLU(lu + 2145), b[167], x);
      x = fma(-CHEM_LDLU(lu + 2146), b[171], x);
      x = fma(-CHEM_LDLU(lu + 2147), b[172], x);
      x = fma(-CHEM_LDLU(lu + 2148), b[173], x);
      x = fma(-CHEM_LDLU(lu + 2149), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2150), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2151), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2152), b[185], x);
      x = fma(-CHEM_LDLU(lu + 2153), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2154), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2155), b[188], x);
      b[164] = x * CHEM_LDLU(vd + 164);
    }
    {
      double x = b[163];
      x = fma(-CHEM_LDLU(lu + 2156), b[166], x);
      x = fma(-CHEM_LDLU(lu + 2157), b[169], x);
      x = fma(-CHEM_LDLU(lu + 2158), b[171], x);
      x = fma(-CHEM_LDLU(lu + 2159), b[172], x);
      x = fma(-CHEM_LDLU(lu + 2160), b[173], x);
      x = fma(-CHEM_LDLU(lu + 2161), b[179], x);
      x = fma(-CHEM_LDLU(lu + 2162), b[180], x);
      x = fma(-CHEM_LDLU(lu + 2163), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2164), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2165), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2166), b[185], x);
      x = fma(-CHEM_LDLU(lu + 2167), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2168), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2169), b[188], x);
      b[163] = x * CHEM_LDLU(vd + 163);
    }
    {
      double x = b[162];
      x = fma(-CHEM_LDLU(lu + 2170), b[171], x);
      x = fma(-CHEM_LDLU(lu + 2171), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2172), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2173), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2174), b[185], x);
      x = fma(-CHEM_LDLU(lu + 2175), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2176), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2177), b[188], x);
      b[162] = x * CHEM_LDLU(vd + 162);
    }
    {
      double x = b[161];
      x = fma(-CHEM_LDLU(lu + 2178), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2179), b[165], x);
      x = fma(-CHEM_LDLU(lu + 2180), b[166], x);
      x = fma(-CHEM_LDLU(lu + 2181), b[173], x);
      x = fma(-CHEM_LDLU(lu + 2182), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2183), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2184), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2185), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2186), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2187), b[188], x);
      b[161] = x * CHEM_LDLU(vd + 161);
    }
    {
      double x = b[160];
      x = fma(-CHEM_LDLU(lu + 2188), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2189), b[166], x);
      x = fma(-CHEM_LDLU(lu + 2190), b[173], x);
      x = fma(-CHEM_LDLU(lu + 2191), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2192), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2193), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2194), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2195), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2196), b[188], x);
      b[160] = x * CHEM_LDLU(vd + 160);
    }
    {
      double x = b[159];
      x = fma(-CHEM_LDLU(lu + 2197), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2198), b[166], x);
      x = fma(-CHEM_LDLU(lu + 2199), b[173], x);
      x = fma(-CHEM_LDLU(lu + 2200), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2201), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2202), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2203), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2204), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2205), b[188], x);
      b[159] = x * CHEM_LDLU(vd + 159);
    }
    {
      double x = b[158];
      x = fma(-CHEM_LDLU(lu + 2206), b[159], x);
      x = fma(-CHEM_LDLU(lu + 2207), b[160], x);
      x = fma(-CHEM_LDLU(lu + 2208), b[161], x);
      x = fma(-CHEM_LDLU(lu + 2209), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2210), b[166], x);
      x = fma(-CHEM_LDLU(lu + 2211), b[169], x);
      x = fma(-CHEM_LDLU(lu + 2212), b[172], x);
      x = fma(-CHEM_LDLU(lu + 2213), b[173], x);
      x = fma(-CHEM_LDLU(lu + 2214), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2215), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2216), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2217), b[185], x);
      x = fma(-CHEM_LDLU(lu + 2218), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2219), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2220), b[188], x);
      b[158] = x * CHEM_LDLU(vd + 158);
    }
    {
      double x = b[157];
      x = fma(-CHEM_LDLU(lu + 2221), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2222), b[164], x);
      x = fma(-CHEM_LDLU(lu + 2223), b[168], x);
      x = fma(-CHEM_LDLU(lu + 2224), b[174], x);
      x = fma(-CHEM_LDLU(lu + 2225), b[180], x);
      x = fma(-CHEM_LDLU(lu + 2226), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2227), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2228), b[183], x);
      x = fma(-CHEM_LDLU(lu + 2229), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2230), b[185], x);
      x = fma(-CHEM_LDLU(lu + 2231), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2232), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2233), b[188], x);
      b[157] = x * CHEM_LDLU(vd + 157);
    }
    {
      double x = b[156];
      x = fma(-CHEM_LDLU(lu + 2234), b[159], x);
      x = fma(-CHEM_LDLU(lu + 2235), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2236), b[166], x);
      x = fma(-CHEM_LDLU(lu + 2237), b[173], x);
      x = fma(-CHEM_LDLU(lu + 2238), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2239), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2240), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2241), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2242), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2243), b[188], x);
      b[156] = x * CHEM_LDLU(vd + 156);
    }
    {
      double x = b[155];
      x = fma(-CHEM_LDLU(lu + 2244), b[156], x);
      x = fma(-CHEM_LDLU(lu + 2245), b[159], x);
      x = fma(-CHEM_LDLU(lu + 2246), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2247), b[166], x);
      x = fma(-CHEM_LDLU(lu + 2248), b[173], x);
      x = fma(-CHEM_LDLU(lu + 2249), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2250), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2251), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2252), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2253), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2254), b[188], x);
      b[155] = x * CHEM_LDLU(vd + 155);
    }
    {
      double x = b[154];
      x = fma(-CHEM_LDLU(lu + 2255), b[155], x);
      x = fma(-CHEM_LDLU(lu + 2256), b[156], x);
      x = fma(-CHEM_LDLU(lu + 2257), b[159], x);
      x = fma(-CHEM_LDLU(lu + 2258), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2259), b[166], x);
      x = fma(-CHEM_LDLU(lu + 2260), b[173], x);
      x = fma(-CHEM_LDLU(lu + 2261), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2262), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2263), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2264), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2265), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2266), b[188], x);
      b[154] = x * CHEM_LDLU(vd + 154);
    }
    {
      double x = b[153];
      x = fma(-CHEM_LDLU(lu + 2267), b[154], x);
      x = fma(-CHEM_LDLU(lu + 2268), b[155], x);
      x = fma(-CHEM_LDLU(lu + 2269), b[156], x);
      x = fma(-CHEM_LDLU(lu + 2270), b[159], x);
      x = fma(-CHEM_LDLU(lu + 2271), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2272), b[166], x);
      x = fma(-CHEM_LDLU(lu + 2273), b[173], x);
      x = fma(-CHEM_LDLU(lu + 2274), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2275), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2276), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2277), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2278), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2279), b[188], x);
      b[153] = x * CHEM_LDLU(vd + 153);
    }
    {
      double x = b[152];
      x = fma(-CHEM_LDLU(lu + 2280), b[153], x);
      x = fma(-CHEM_LDLU(lu + 2281), b[154], x);
      x = fma(-CHEM_LDLU(lu + 2282), b[155], x);
      x = fma(-CHEM_LDLU(lu + 2283), b[156], x);
      x = fma(-CHEM_LDLU(lu + 2284), b[159], x);
      x = fma(-CHEM_LDLU(lu + 2285), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2286), b[166], x);
      x = fma(-CHEM_LDLU(lu + 2287), b[173], x);
      x = fma(-CHEM_LDLU(lu + 2288), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2289), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2290), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2291), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2292), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2293), b[188], x);
      b[152] = x * CHEM_LDLU(vd + 152);
    }
    {
      double x = b[151];
      x = fma(-CHEM_LDLU(lu + 2294), b[152], x);
      x = fma(-CHEM_LDLU(lu + 2295), b[154], x);
      x = fma(-CHEM_LDLU(lu + 2296), b[155], x);
      x = fma(-CHEM_LDLU(lu + 2297), b[156], x);
      x = fma(-CHEM_LDLU(lu + 2298), b[159], x);
      x = fma(-CHEM_LDLU(lu + 2299), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2300), b[166], x);
      x = fma(-CHEM_LDLU(lu + 2301), b[173], x);
      x = fma(-CHEM_LDLU(lu + 2302), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2303), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2304), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2305), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2306), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2307), b[188], x);
      b[151] = x * CHEM_LDLU(vd + 151);
    }
    {
      double x = b[150];
      x = fma(-CHEM_LDLU(lu + 2308), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2309), b[163], x);
      x = fma(-CHEM_LDLU(lu + 2310), b[171], x);
      x = fma(-CHEM_LDLU(lu + 2311), b[180], x);
      x = fma(-CHEM_LDLU(lu + 2312), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2313), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2314), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2315), b[185], x);
      x = fma(-CHEM_LDLU(lu + 2316), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2317), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2318), b[188], x);
      b[150] = x * CHEM_LDLU(vd + 150);
    }
    {
      double x = b[149];
      x = fma(-CHEM_LDLU(lu + 2319), b[151], x);
      x = fma(-CHEM_LDLU(lu + 2320), b[152], x);
      x = fma(-CHEM_LDLU(lu + 2321), b[153], x);
      x = fma(-CHEM_LDLU(lu + 2322), b[154], x);
      x = fma(-CHEM_LDLU(lu + 2323), b[155], x);
      x = fma(-CHEM_LDLU(lu + 2324), b[156], x);
      x = fma(-CHEM_LDLU(lu + 2325), b[159], x);
      x = fma(-CHEM_LDLU(lu + 2326), b[166], x);
      x = fma(-CHEM_LDLU(lu + 2327), b[173], x);
      x = fma(-CHEM_LDLU(lu + 2328), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2329), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2330), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2331), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2332), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2333), b[188], x);
      b[149] = x * CHEM_LDLU(vd + 149);
    }
    {
      double x = b[148];
      x = fma(-CHEM_LDLU(lu + 2334), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2335), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2336), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2337), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2338), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2339), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2340), b[188], x);
      b[148] = x * CHEM_LDLU(vd + 148);
    }
    {
      double x = b[147];
      x = fma(-CHEM_LDLU(lu + 2341), b[151], x);
      x = fma(-CHEM_LDLU(lu + 2342), b[152], x);
      x = fma(-CHEM_LDLU(lu + 2343), b[154], x);
      x = fma(-CHEM_LDLU(lu + 2344), b[155], x);
      x = fma(-CHEM_LDLU(lu + 2345), b[156], x);
      x = fma(-CHEM_LDLU(lu + 2346), b[159], x);
      x = fma(-CHEM_LDLU(lu + 2347), b[166], x);
      x = fma(-CHEM_LDLU(lu + 2348), b[173], x);
      x = fma(-CHEM_LDLU(lu + 2349), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2350), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2351), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2352), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2353), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2354), b[188], x);
      b[147] = x * CHEM_LDLU(vd + 147);
    }
    {
      double x = b[146];
      x = fma(-CHEM_LDLU(lu + 2355), b[148], x);
      x = fma(-CHEM_LDLU(lu + 2356), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2357), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2358), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2359), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2360), b[185], x);
      x = fma(-CHEM_LDLU(lu + 2361), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2362), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2363), b[188], x);
      b[146] = x * CHEM_LDLU(vd + 146);
    }
    {
      double x = b[145];
      x = fma(-CHEM_LDLU(lu + 2364), b[147], x);
      x = fma(-CHEM_LDLU(lu + 2365), b[151], x);
      x = fma(-CHEM_LDLU(lu + 2366), b[152], x);
      x = fma(-CHEM_LDLU(lu + 2367), b[154], x);
      x = fma(-CHEM_LDLU(lu + 2368), b[155], x);
      x = fma(-CHEM_LDLU(lu + 2369), b[156], x);
      x = fma(-CHEM_LDLU(lu + 2370), b[159], x);
      x = fma(-CHEM_LDLU(lu + 2371), b[166], x);
      x = fma(-CHEM_LDLU(lu + 2372), b[173], x);
      x = fma(-CHEM_LDLU(lu + 2373), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2374), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2375), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2376), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2377), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2378), b[188], x);
      b[145] = x * CHEM_LDLU(vd + 145);
    }
    {
      double x = b[144];
      x = fma(-CHEM_LDLU(lu + 2379), b[145], x);
      x = fma(-CHEM_LDLU(lu + 2380), b[147], x);
      x = fma(-CHEM_LDLU(lu + 2381), b[151], x);
      x = fma(-CHEM_LDLU(lu + 2382), b[152], x);
      x = fma(-CHEM_LDLU(lu + 2383), b[155], x);
      x = fma(-CHEM_LDLU(lu + 2384), b[156], x);
      x = fma(-CHEM_LDLU(lu + 2385), b[159], x);
      x = fma(-CHEM_LDLU(lu + 2386), b[166], x);
      x = fma(-CHEM_LDLU(lu + 2387), b[173], x);
      x = fma(-CHEM_LDLU(lu + 2388), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2389), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2390), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2391), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2392), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2393), b[188], x);
      b[144] = x * CHEM_LDLU(vd + 144);
    }
    {
      double x = b[143];
      x = fma(-CHEM_LDLU(lu + 2394), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2395), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2396), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2397), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2398), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2399), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2400), b[188], x);
      b[143] = x * CHEM_LDLU(vd + 143);
    }
    {
      double x = b[142];
      x = fma(-CHEM_LDLU(lu + 2401), b[143], x);
      x = fma(-CHEM_LDLU(lu + 2402), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2403), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2404), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2405), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2406), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2407), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2408), b[188], x);
      b[142] = x * CHEM_LDLU(vd + 142);
    }
    {
      double x = b[141];
      x = fma(-CHEM_LDLU(lu + 2409), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2410), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2411), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2412), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2413), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2414), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2415), b[188], x);
      b[141] = x * CHEM_LDLU(vd + 141);
    }
    {
      double x = b[140];
      x = fma(-CHEM_LDLU(lu + 2416), b[160], x);
      x = fma(-CHEM_LDLU(lu + 2417), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2418), b[169], x);
      x = fma(-CHEM_LDLU(lu + 2419), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2420), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2421), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2422), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2423), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2424), b[188], x);
      b[140] = x * CHEM_LDLU(vd + 140);
    }
    {
      double x = b[139];
      x = fma(-CHEM_LDLU(lu + 2425), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2426), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2427), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2428), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2429), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2430), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2431), b[188], x);
      b[139] = x * CHEM_LDLU(vd + 139);
    }
    {
      double x = b[138];
      x = fma(-CHEM_LDLU(lu + 2432), b[147], x);
      x = fma(-CHEM_LDLU(lu + 2433), b[151], x);
      x = fma(-CHEM_LDLU(lu + 2434), b[155], x);
      x = fma(-CHEM_LDLU(lu + 2435), b[159], x);
      x = fma(-CHEM_LDLU(lu + 2436), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2437), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2438), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2439), b[188], x);
      b[138] = x * CHEM_LDLU(vd + 138);
    }
    {
      double x = b[137];
      x = fma(-CHEM_LDLU(lu + 2440), b[142], x);
      x = fma(-CHEM_LDLU(lu + 2441), b[143], x);
      x = fma(-CHEM_LDLU(lu + 2442), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2443), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2444), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2445), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2446), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2447), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2448), b[188], x);
      b[137] = x * CHEM_LDLU(vd + 137);
    }
    {
      double x = b[136];
      x = fma(-CHEM_LDLU(lu + 2449), b[137], x);
      x = fma(-CHEM_LDLU(lu + 2450), b[143], x);
      x = fma(-CHEM_LDLU(lu + 2451), b[148], x);
      x = fma(-CHEM_LDLU(lu + 2452), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2453), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2454), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2455), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2456), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2457), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2458), b[188], x);
      b[136] = x * CHEM_LDLU(vd + 136);
    }
    {
      double x = b[135];
      x = fma(-CHEM_LDLU(lu + 2459), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2460), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2461), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2462), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2463), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2464), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2465), b[188], x);
      b[135] = x * CHEM_LDLU(vd + 135);
    }
    {
      double x = b[134];
      x = fma(-CHEM_LDLU(lu + 2466), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2467), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2468), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2469), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2470), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2471), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2472), b[188], x);
      b[134] = x * CHEM_LDLU(vd + 134);
    }
    {
      double x = b[133];
      x = fma(-CHEM_LDLU(lu + 2473), b[134], x);
      x = fma(-CHEM_LDLU(lu + 2474), b[142], x);
      x = fma(-CHEM_LDLU(lu + 2475), b[143], x);
      x = fma(-CHEM_LDLU(lu + 2476), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2477), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2478), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2479), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2480), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2481), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2482), b[188], x);
      b[133] = x * CHEM_LDLU(vd + 133);
    }
    {
      double x = b[132];
      x = fma(-CHEM_LDLU(lu + 2483), b[138], x);
      x = fma(-CHEM_LDLU(lu + 2484), b[145], x);
      x = fma(-CHEM_LDLU(lu + 2485), b[147], x);
      x = fma(-CHEM_LDLU(lu + 2486), b[151], x);
      x = fma(-CHEM_LDLU(lu + 2487), b[155], x);
      x = fma(-CHEM_LDLU(lu + 2488), b[156], x);
      x = fma(-CHEM_LDLU(lu + 2489), b[159], x);
      x = fma(-CHEM_LDLU(lu + 2490), b[166], x);
      x = fma(-CHEM_LDLU(lu + 2491), b[173], x);
      x = fma(-CHEM_LDLU(lu + 2492), b[188], x);
      b[132] = x * CHEM_LDLU(vd + 132);
    }
    {
      double x = b[131];
      x = fma(-CHEM_LDLU(lu + 2493), b[134], x);
      x = fma(-CHEM_LDLU(lu + 2494), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2495), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2496), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2497), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2498), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2499), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2500), b[188], x);
      b[131] = x * CHEM_LDLU(vd + 131);
    }
    {
      double x = b[130];
      x = fma(-CHEM_LDLU(lu + 2501), b[131], x);
      x = fma(-CHEM_LDLU(lu + 2502), b[134], x);
      x = fma(-CHEM_LDLU(lu + 2503), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2504), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2505), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2506), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2507), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2508), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2509), b[188], x);
      b[130] = x * CHEM_LDLU(vd + 130);
    }
    {
      double x = b[129];
      x = fma(-CHEM_LDLU(lu + 2510), b[134], x);
      x = fma(-CHEM_LDLU(lu + 2511), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2512), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2513), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2514), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2515), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2516), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2517), b[188], x);
      b[129] = x * CHEM_LDLU(vd + 129);
    }
    {
      double x = b[128];
      x = fma(-CHEM_LDLU(lu + 2518), b[130], x);
      x = fma(-CHEM_LDLU(lu + 2519), b[131], x);
      x = fma(-CHEM_LDLU(lu + 2520), b[142], x);
      x = fma(-CHEM_LDLU(lu + 2521), b[143], x);
      x = fma(-CHEM_LDLU(lu + 2522), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2523), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2524), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2525), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2526), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2527), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2528), b[188], x);
      b[128] = x * CHEM_LDLU(vd + 128);
    }
    {
      double x = b[127];
      x = fma(-CHEM_LDLU(lu + 2529), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2530), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2531), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2532), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2533), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2534), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2535), b[188], x);
      b[127] = x * CHEM_LDLU(vd + 127);
    }
    {
      double x = b[126];
      x = fma(-CHEM_LDLU(lu + 2536), b[127], x);
      x = fma(-CHEM_LDLU(lu + 2537), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2538), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2539), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2540), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2541), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2542), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2543), b[188], x);
      b[126] = x * CHEM_LDLU(vd + 126);
    }
    {
      double x = b[125];
      x = fma(-CHEM_LDLU(lu + 2544), b[143], x);
      x = fma(-CHEM_LDLU(lu + 2545), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2546), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2547), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2548), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2549), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2550), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2551), b[188], x);
      b[125] = x * CHEM_LDLU(vd + 125);
    }
    {
      double x = b[124];
      x = fma(-CHEM_LDLU(lu + 2552), b[132], x);
      x = fma(-CHEM_LDLU(lu + 2553), b[138], x);
      x = fma(-CHEM_LDLU(lu + 2554), b[147], x);
      x = fma(-CHEM_LDLU(lu + 2555), b[151], x);
      x = fma(-CHEM_LDLU(lu + 2556), b[155], x);
      x = fma(-CHEM_LDLU(lu + 2557), b[159], x);
      x = fma(-CHEM_LDLU(lu + 2558), b[166], x);
      x = fma(-CHEM_LDLU(lu + 2559), b[173], x);
      x = fma(-CHEM_LDLU(lu + 2560), b[188], x);
      b[124] = x * CHEM_LDLU(vd + 124);
    }
    {
      double x = b[123];
      x = fma(-CHEM_LDLU(lu + 2561), b[130], x);
      x = fma(-CHEM_LDLU(lu + 2562), b[131], x);
      x = fma(-CHEM_LDLU(lu + 2563), b[134], x);
      x = fma(-CHEM_LDLU(lu + 2564), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2565), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2566), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2567), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2568), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2569), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2570), b[188], x);
      b[123] = x * CHEM_LDLU(vd + 123);
    }
    {
      double x = b[122];
      x = fma(-CHEM_LDLU(lu + 2571), b[128], x);
      x = fma(-CHEM_LDLU(lu + 2572), b[142], x);
      x = fma(-CHEM_LDLU(lu + 2573), b[143], x);
      x = fma(-CHEM_LDLU(lu + 2574), b[144], x);
      x = fma(-CHEM_LDLU(lu + 2575), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2576), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2577), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2578), b[188], x);
      b[122] = x * CHEM_LDLU(vd + 122);
    }
    {
      double x = b[121];
      x = fma(-CHEM_LDLU(lu + 2579), b[137], x);
      x = fma(-CHEM_LDLU(lu + 2580), b[148], x);
      x = fma(-CHEM_LDLU(lu + 2581), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2582), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2583), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2584), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2585), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2586), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2587), b[188], x);
      b[121] = x * CHEM_LDLU(vd + 121);
    }
    {
      double x = b[120];
      x = fma(-CHEM_LDLU(lu + 2588), b[130], x);
      x = fma(-CHEM_LDLU(lu + 2589), b[131], x);
      x = fma(-CHEM_LDLU(lu + 2590), b[134], x);
      x = fma(-CHEM_LDLU(lu + 2591), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2592), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2593), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2594), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2595), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2596), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2597), b[188], x);
      b[120] = x * CHEM_LDLU(vd + 120);
    }
    {
      double x = b[119];
      x = fma(-CHEM_LDLU(lu + 2598), b[139], x);
      x = fma(-CHEM_LDLU(lu + 2599), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2600), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2601), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2602), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2603), b[185], x);
      x = fma(-CHEM_LDLU(lu + 2604), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2605), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2606), b[188], x);
      b[119] = x * CHEM_LDLU(vd + 119);
    }
    {
      double x = b[118];
      x = fma(-CHEM_LDLU(lu + 2607), b[152], x);
      x = fma(-CHEM_LDLU(lu + 2608), b[154], x);
      x = fma(-CHEM_LDLU(lu + 2609), b[172], x);
      x = fma(-CHEM_LDLU(lu + 2610), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2611), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2612), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2613), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2614), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2615), b[188], x);
      b[118] = x * CHEM_LDLU(vd + 118);
    }
    {
      double x = b[117];
      x = fma(-CHEM_LDLU(lu + 2616), b[130], x);
      x = fma(-CHEM_LDLU(lu + 2617), b[131], x);
      x = fma(-CHEM_LDLU(lu + 2618), b[134], x);
      x = fma(-CHEM_LDLU(lu + 2619), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2620), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2621), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2622), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2623), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2624), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2625), b[188], x);
      b[117] = x * CHEM_LDLU(vd + 117);
    }
    {
      double x = b[116];
      x = fma(-CHEM_LDLU(lu + 2626), b[130], x);
      x = fma(-CHEM_LDLU(lu + 2627), b[131], x);
      x = fma(-CHEM_LDLU(lu + 2628), b[134], x);
      x = fma(-CHEM_LDLU(lu + 2629), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2630), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2631), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2632), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2633), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2634), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2635), b[188], x);
      b[116] = x * CHEM_LDLU(vd + 116);
    }
    {
      double x = b[115];
      x = fma(-CHEM_LDLU(lu + 2636), b[143], x);
      x = fma(-CHEM_LDLU(lu + 2637), b[150], x);
      x = fma(-CHEM_LDLU(lu + 2638), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2639), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2640), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2641), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2642), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2643), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2644), b[188], x);
      b[115] = x * CHEM_LDLU(vd + 115);
    }
    {
      double x = b[114];
      x = fma(-CHEM_LDLU(lu + 2645), b[139], x);
      x = fma(-CHEM_LDLU(lu + 2646), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2647), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2648), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2649), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2650), b[185], x);
      x = fma(-CHEM_LDLU(lu + 2651), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2652), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2653), b[188], x);
      b[114] = x * CHEM_LDLU(vd + 114);
    }
    {
      double x = b[113];
      x = fma(-CHEM_LDLU(lu + 2654), b[139], x);
      x = fma(-CHEM_LDLU(lu + 2655), b[141], x);
      x = fma(-CHEM_LDLU(lu + 2656), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2657), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2658), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2659), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2660), b[185], x);
      x = fma(-CHEM_LDLU(lu + 2661), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2662), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2663), b[188], x);
      b[113] = x * CHEM_LDLU(vd + 113);
    }
    {
      double x = b[112];
      x = fma(-CHEM_LDLU(lu + 2664), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2665), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2666), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2667), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2668), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2669), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2670), b[188], x);
      b[112] = x * CHEM_LDLU(vd + 112);
    }
    {
      double x = b[111];
      x = fma(-CHEM_LDLU(lu + 2671), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2672), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2673), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2674), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2675), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2676), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2677), b[188], x);
      b[111] = x * CHEM_LDLU(vd + 111);
    }
    {
      double x = b[110];
      x = fma(-CHEM_LDLU(lu + 2678), b[111], x);
      x = fma(-CHEM_LDLU(lu + 2679), b[129], x);
      x = fma(-CHEM_LDLU(lu + 2680), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2681), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2682), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2683), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2684), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2685), b[188], x);
      b[110] = x * CHEM_LDLU(vd + 110);
    }
    {
      double x = b[109];
      x = fma(-CHEM_LDLU(lu + 2686), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2687), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2688), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2689), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2690), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2691), b[188], x);
      b[109] = x * CHEM_LDLU(vd + 109);
    }
    {
      double x = b[108];
      x = fma(-CHEM_LDLU(lu + 2692), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2693), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2694), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2695), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2696), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2697), b[188], x);
      b[108] = x * CHEM_LDLU(vd + 108);
    }
    {
      double x = b[107];
      x = fma(-CHEM_LDLU(lu + 2698), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2699), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2700), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2701), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2702), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2703), b[188], x);
      b[107] = x * CHEM_LDLU(vd + 107);
    }
    {
      double x = b[106];
      x = fma(-CHEM_LDLU(lu + 2704), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2705), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2706), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2707), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2708), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2709), b[188], x);
      b[106] = x * CHEM_LDLU(vd + 106);
    }
    {
      double x = b[105];
      x = fma(-CHEM_LDLU(lu + 2710), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2711), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2712), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2713), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2714), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2715), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2716), b[188], x);
      b[105] = x * CHEM_LDLU(vd + 105);
    }
    {
      double x = b[104];
      x = fma(-CHEM_LDLU(lu + 2717), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2718), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2719), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2720), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2721), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2722), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2723), b[188], x);
      b[104] = x * CHEM_LDLU(vd + 104);
    }
    {
      double x = b[103];
      x = fma(-CHEM_LDLU(lu + 2724), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2725), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2726), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2727), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2728), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2729), b[188], x);
      b[103] = x * CHEM_LDLU(vd + 103);
    }
    {
      double x = b[102];
      x = fma(-CHEM_LDLU(lu + 2730), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2731), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2732), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2733), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2734), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2735), b[188], x);
      b[102] = x * CHEM_LDLU(vd + 102);
    }
    {
      double x = b[101];
      x = fma(-CHEM_LDLU(lu + 2736), b[139], x);
      x = fma(-CHEM_LDLU(lu + 2737), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2738), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2739), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2740), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2741), b[185], x);
      x = fma(-CHEM_LDLU(lu + 2742), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2743), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2744), b[188], x);
      b[101] = x * CHEM_LDLU(vd + 101);
    }
    {
      double x = b[100];
      x = fma(-CHEM_LDLU(lu + 2745), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2746), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2747), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2748), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2749), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2750), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2751), b[188], x);
      b[100] = x * CHEM_LDLU(vd + 100);
    }
    {
      double x = b[99];
      x = fma(-CHEM_LDLU(lu + 2752), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2753), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2754), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2755), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2756), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2757), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2758), b[188], x);
      b[99] = x * CHEM_LDLU(vd + 99);
    }
    {
      double x = b[98];
      x = fma(-CHEM_LDLU(lu + 2759), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2760), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2761), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2762), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2763), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2764), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2765), b[188], x);
      b[98] = x * CHEM_LDLU(vd + 98);
    }
    {
      double x = b[97];
      x = fma(-CHEM_LDLU(lu + 2766), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2767), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2768), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2769), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2770), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2771), b[188], x);
      b[97] = x * CHEM_LDLU(vd + 97);
    }
    {
      double x = b[96];
      x = fma(-CHEM_LDLU(lu + 2772), b[98], x);
      x = fma(-CHEM_LDLU(lu + 2773), b[101], x);
      x = fma(-CHEM_LDLU(lu + 2774), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2775), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2776), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2777), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2778), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2779), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2780), b[188], x);
      b[96] = x * CHEM_LDLU(vd + 96);
    }
    {
      double x = b[95];
      x = fma(-CHEM_LDLU(lu + 2781), b[119], x);
      x = fma(-CHEM_LDLU(lu + 2782), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2783), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2784), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2785), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2786), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2787), b[187], x);
      b[95] = x * CHEM_LDLU(vd + 95);
    }
    {
      double x = b[94];
      x = fma(-CHEM_LDLU(lu + 2788), b[111], x);
      x = fma(-CHEM_LDLU(lu + 2789), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2790), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2791), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2792), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2793), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2794), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2795), b[188], x);
      b[94] = x * CHEM_LDLU(vd + 94);
    }
    {
      double x = b[93];
      x = fma(-CHEM_LDLU(lu + 2796), b[178], x);
      x = fma(-CHEM_LDLU(lu + 2797), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2798), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2799), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2800), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2801), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2802), b[188], x);
      b[93] = x * CHEM_LDLU(vd + 93);
    }
    {
      double x = b[92];
      x = fma(-CHEM_LDLU(lu + 2803), b[101], x);
      x = fma(-CHEM_LDLU(lu + 2804), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2805), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2806), b[188], x);
      b[92] = x * CHEM_LDLU(vd + 92);
    }
    {
      double x = b[91];
      x = fma(-CHEM_LDLU(lu + 2807), b[121], x);
      x = fma(-CHEM_LDLU(lu + 2808), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2809), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2810), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2811), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2812), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2813), b[188], x);
      b[91] = x * CHEM_LDLU(vd + 91);
    }
    {
      double x = b[90];
      x = fma(-CHEM_LDLU(lu + 2814), b[148], x);
      x = fma(-CHEM_LDLU(lu + 2815), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2816), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2817), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2818), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2819), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2820), b[188], x);
      b[90] = x * CHEM_LDLU(vd + 90);
    }
    {
      double x = b[89];
      x = fma(-CHEM_LDLU(lu + 2821), b[140], x);
      x = fma(-CHEM_LDLU(lu + 2822), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2823), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2824), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2825), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2826), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2827), b[188], x);
      b[89] = x * CHEM_LDLU(vd + 89);
    }
    {
      double x = b[88];
      x = fma(-CHEM_LDLU(lu + 2828), b[143], x);
      x = fma(-CHEM_LDLU(lu + 2829), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2830), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2831), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2832), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2833), b[188], x);
      b[88] = x * CHEM_LDLU(vd + 88);
    }
    {
      double x = b[87];
      x = fma(-CHEM_LDLU(lu + 2834), b[134], x);
      x = fma(-CHEM_LDLU(lu + 2835), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2836), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2837), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2838), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2839), b[188], x);
      b[87] = x * CHEM_LDLU(vd + 87);
    }
    {
      double x = b[86];
      x = fma(-CHEM_LDLU(lu + 2840), b[98], x);
      x = fma(-CHEM_LDLU(lu + 2841), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2842), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2843), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2844), b[188], x);
      b[86] = x * CHEM_LDLU(vd + 86);
    }
    {
      double x = b[85];
      x = fma(-CHEM_LDLU(lu + 2845), b[116], x);
      x = fma(-CHEM_LDLU(lu + 2846), b[117], x);
      x = fma(-CHEM_LDLU(lu + 2847), b[120], x);
      x = fma(-CHEM_LDLU(lu + 2848), b[123], x);
      x = fma(-CHEM_LDLU(lu + 2849), b[130], x);
      x = fma(-CHEM_LDLU(lu + 2850), b[131], x);
      x = fma(-CHEM_LDLU(lu + 2851), b[134], x);
      b[85] = x * CHEM_LDLU(vd + 85);
    }
    {
      double x = b[84];
      x = fma(-CHEM_LDLU(lu + 2852), b[139], x);
      x = fma(-CHEM_LDLU(lu + 2853), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2854), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2855), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2856), b[185], x);
      x = fma(-CHEM_LDLU(lu + 2857), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2858), b[188], x);
      b[84] = x * CHEM_LDLU(vd + 84);
    }
}
__device__ __noinline__ void solve_s1_0_4(double* __restrict__ ws, int rhs)
{
    const double* __restrict__ lu = ws + 3484;
    const double* __restrict__ vd = ws + 6769;
    double* __restrict__ b = ws + rhs;
    (void)vd;
    {
      double x = b[83];
      x = fma(-CHEM_LDLU(lu + 2859), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2860), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2861), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2862), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2863), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2864), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2865), b[188], x);
      b[83] = x * CHEM_LDLU(vd + 83);
    }
    {
      double x = b[82];
      x = fma(-CHEM_LDLU(lu + 2866), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2867), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2868), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2869), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2870), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2871), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2872), b[188], x);
      b[82] = x * CHEM_LDLU(vd + 82);
    }
    {
      double x = b[81];
      x = fma(-CHEM_LDLU(lu + 2873), b[139], x);
      x = fma(-CHEM_LDLU(lu + 2874), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2875), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2876), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2877), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2878), b[188], x);
      b[81] = x * CHEM_LDLU(vd + 81);
    }
    {
      double x = b[80];
      x = fma(-CHEM_LDLU(lu + 2879), b[142], x);
      x = fma(-CHEM_LDLU(lu + 2880), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2881), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2882), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2883), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2884), b[188], x);
      b[80] = x * CHEM_LDLU(vd + 80);
    }
    {
      double x = b[79];
      x = fma(-CHEM_LDLU(lu + 2885), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2886), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2887), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2888), b[188], x);
      b[79] = x * CHEM_LDLU(vd + 79);
    }
    {
      double x = b[78];
      x = fma(-CHEM_LDLU(lu + 2889), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2890), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2891), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2892), b[188], x);
      b[78] = x * CHEM_LDLU(vd + 78);
    }
    {
      double x = b[77];
      x = fma(-CHEM_LDLU(lu + 2893), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2894), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2895), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2896), b[188], x);
      b[77] = x * CHEM_LDLU(vd + 77);
    }
    {
      double x = b[76];
      x = fma(-CHEM_LDLU(lu + 2897), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2898), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2899), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2900), b[188], x);
      b[76] = x * CHEM_LDLU(vd + 76);
    }
    {
      double x = b[75];
      x = fma(-CHEM_LDLU(lu + 2901), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2902), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2903), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2904), b[188], x);
      b[75] = x * CHEM_LDLU(vd + 75);
    }
    {
      double x = b[74];
      x = fma(-CHEM_LDLU(lu + 2905), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2906), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2907), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2908), b[188], x);
      b[74] = x * CHEM_LDLU(vd + 74);
    }
    {
      double x = b[73];
      x = fma(-CHEM_LDLU(lu + 2909), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2910), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2911), b[185], x);
      x = fma(-CHEM_LDLU(lu + 2912), b[186], x);
      b[73] = x * CHEM_LDLU(vd + 73);
    }
    {
      double x = b[72];
      x = fma(-CHEM_LDLU(lu + 2913), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2914), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2915), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2916), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2917), b[188], x);
      b[72] = x * CHEM_LDLU(vd + 72);
    }
    {
      double x = b[71];
      x = fma(-CHEM_LDLU(lu + 2918), b[81], x);
      x = fma(-CHEM_LDLU(lu + 2919), b[181], x);
      x = fma(-CHEM_LDLU(lu + 2920), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2921), b[184], x);
      x = fma(-CHEM_LDLU(lu + 2922), b[186], x);
      b[71] = x * CHEM_LDLU(vd + 71);
    }
    {
      double x = b[70];
      x = fma(-CHEM_LDLU(lu + 2923), b[111], x);
      x = fma(-CHEM_LDLU(lu + 2924), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2925), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2926), b[188], x);
      b[70] = x * CHEM_LDLU(vd + 70);
    }
    {
      double x = b[69];
      x = fma(-CHEM_LDLU(lu + 2927), b[87], x);
      x = fma(-CHEM_LDLU(lu + 2928), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2929), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2930), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2931), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2932), b[188], x);
      b[69] = x * CHEM_LDLU(vd + 69);
    }
    {
      double x = b[68];
      x = fma(-CHEM_LDLU(lu + 2933), b[86], x);
      x = fma(-CHEM_LDLU(lu + 2934), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2935), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2936), b[188], x);
      b[68] = x * CHEM_LDLU(vd + 68);
    }
    {
      double x = b[67];
      x = fma(-CHEM_LDLU(lu + 2937), b[122], x);
      x = fma(-CHEM_LDLU(lu + 2938), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2939), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2940), b[187], x);
      b[67] = x * CHEM_LDLU(vd + 67);
    }
    {
      double x = b[66];
      x = fma(-CHEM_LDLU(lu + 2941), b[79], x);
      x = fma(-CHEM_LDLU(lu + 2942), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2943), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2944), b[187], x);
      b[66] = x * CHEM_LDLU(vd + 66);
    }
    {
      double x = b[65];
      x = fma(-CHEM_LDLU(lu + 2945), b[78], x);
      x = fma(-CHEM_LDLU(lu + 2946), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2947), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2948), b[187], x);
      b[65] = x * CHEM_LDLU(vd + 65);
    }
    {
      double x = b[64];
      x = fma(-CHEM_LDLU(lu + 2949), b[77], x);
      x = fma(-CHEM_LDLU(lu + 2950), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2951), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2952), b[187], x);
      b[64] = x * CHEM_LDLU(vd + 64);
    }
    {
      double x = b[63];
      x = fma(-CHEM_LDLU(lu + 2953), b[76], x);
      x = fma(-CHEM_LDLU(lu + 2954), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2955), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2956), b[187], x);
      b[63] = x * CHEM_LDLU(vd + 63);
    }
    {
      double x = b[62];
      x = fma(-CHEM_LDLU(lu + 2957), b[75], x);
      x = fma(-CHEM_LDLU(lu + 2958), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2959), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2960), b[187], x);
      b[62] = x * CHEM_LDLU(vd + 62);
    }
    {
      double x = b[61];
      x = fma(-CHEM_LDLU(lu + 2961), b[74], x);
      x = fma(-CHEM_LDLU(lu + 2962), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2963), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2964), b[187], x);
      b[61] = x * CHEM_LDLU(vd + 61);
    }
    {
      double x = b[60];
      x = fma(-CHEM_LDLU(lu + 2965), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2966), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2967), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2968), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2969), b[188], x);
      b[60] = x * CHEM_LDLU(vd + 60);
    }
    {
      double x = b[59];
      x = fma(-CHEM_LDLU(lu + 2970), b[86], x);
      x = fma(-CHEM_LDLU(lu + 2971), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2972), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2973), b[188], x);
      b[59] = x * CHEM_LDLU(vd + 59);
    }
    {
      double x = b[58];
      x = fma(-CHEM_LDLU(lu + 2974), b[99], x);
      x = fma(-CHEM_LDLU(lu + 2975), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2976), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2977), b[188], x);
      b[58] = x * CHEM_LDLU(vd + 58);
    }
    {
      double x = b[57];
      x = fma(-CHEM_LDLU(lu + 2978), b[146], x);
      x = fma(-CHEM_LDLU(lu + 2979), b[185], x);
      x = fma(-CHEM_LDLU(lu + 2980), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2981), b[188], x);
      b[57] = x * CHEM_LDLU(vd + 57);
    }
    {
      double x = b[56];
      x = fma(-CHEM_LDLU(lu + 2982), b[110], x);
      x = fma(-CHEM_LDLU(lu + 2983), b[146], x);
      x = fma(-CHEM_LDLU(lu + 2984), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2985), b[188], x);
      b[56] = x * CHEM_LDLU(vd + 56);
    }
    {
      double x = b[55];
      x = fma(-CHEM_LDLU(lu + 2986), b[86], x);
      x = fma(-CHEM_LDLU(lu + 2987), b[92], x);
      x = fma(-CHEM_LDLU(lu + 2988), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2989), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2990), b[188], x);
      b[55] = x * CHEM_LDLU(vd + 55);
    }
    {
      double x = b[54];
      x = fma(-CHEM_LDLU(lu + 2991), b[143], x);
      x = fma(-CHEM_LDLU(lu + 2992), b[182], x);
      x = fma(-CHEM_LDLU(lu + 2993), b[187], x);
      x = fma(-CHEM_LDLU(lu + 2994), b[188], x);
      b[54] = x * CHEM_LDLU(vd + 54);
    }
    {
      double x = b[53];
      x = fma(-CHEM_LDLU(lu + 2995), b[137], x);
      x = fma(-CHEM_LDLU(lu + 2996), b[162], x);
      x = fma(-CHEM_LDLU(lu + 2997), b[186], x);
      x = fma(-CHEM_LDLU(lu + 2998), b[188], x);
      b[53] = x * CHEM_LDLU(vd + 53);
    }
    {
      double x = b[52];
      x = fma(-CHEM_LDLU(lu + 2999), b[134], x);
      x = fma(-CHEM_LDLU(lu + 3000), b[162], x);
      x = fma(-CHEM_LDLU(lu + 3001), b[182], x);
      x = fma(-CHEM_LDLU(lu + 3002), b[186], x);
      x = fma(-CHEM_LDLU(lu + 3003), b[187], x);
      x = fma(-CHEM_LDLU(lu + 3004), b[188], x);
      b[52] = x * CHEM_LDLU(vd + 52);
    }
    {
      double x = b[51];
      x = fma(-CHEM_LDLU(lu + 3005), b[162], x);
      x = fma(-CHEM_LDLU(lu + 3006), b[182], x);
      x = fma(-CHEM_LDLU(lu + 3007), b[186], x);
      x = fma(-CHEM_LDLU(lu + 3008), b[187], x);
      x = fma(-CHEM_LDLU(lu + 3009), b[188], x);
      b[51] = x * CHEM_LDLU(vd + 51);
    }
    {
      double x = b[50];
      x = fma(-CHEM_LDLU(lu + 3010), b[162], x);
      x = fma(-CHEM_LDLU(lu + 3011), b[186], x);
      x = fma(-CHEM_LDLU(lu + 3012), b[188], x);
      b[50] = x * CHEM_LDLU(vd + 50);
    }
    {
      double x = b[49];
      x = fma(-CHEM_LDLU(lu + 3013), b[162], x);
      x = fma(-CHEM_LDLU(lu + 3014), b[186], x);
      x = fma(-CHEM_LDLU(lu + 3015), b[188], x);
      b[49] = x * CHEM_LDLU(vd + 49);
    }
    {
      double x = b[48];
      x = fma(-CHEM_LDLU(lu + 3016), b[150], x);
      x = fma(-CHEM_LDLU(lu + 3017), b[185], x);
      x = fma(-CHEM_LDLU(lu + 3018), b[188], x);
      b[48] = x * CHEM_LDLU(vd + 48);
    }
    {
      double x = b[47];
      x = fma(-CHEM_LDLU(lu + 3019), b[94], x);
      x = fma(-CHEM_LDLU(lu + 3020), b[184], x);
      x = fma(-CHEM_LDLU(lu + 3021), b[188], x);
      b[47] = x * CHEM_LDLU(vd + 47);
    }
    {
      double x = b[46];
      x = fma(-CHEM_LDLU(lu + 3022), b[176], x);
      x = fma(-CHEM_LDLU(lu + 3023), b[184], x);
      x = fma(-CHEM_LDLU(lu + 3024), b[188], x);
      b[46] = x * CHEM_LDLU(vd + 46);
    }
    {
      double x = b[45];
      x = fma(-CHEM_LDLU(lu + 3025), b[162], x);
      x = fma(-CHEM_LDLU(lu + 3026), b[186], x);
      x = fma(-CHEM_LDLU(lu + 3027), b[188], x);
      b[45] = x * CHEM_LDLU(vd + 45);
    }
    {
      double x = b[44];
      x = fma(-CHEM_LDLU(lu + 3028), b[162], x);
      x = fma(-CHEM_LDLU(lu + 3029), b[186], x);
      x = fma(-CHEM_LDLU(lu + 3030), b[188], x);
      b[44] = x * CHEM_LDLU(vd + 44);
    }
    {
      double x = b[43];
      x = fma(-CHEM_LDLU(lu + 3031), b[87], x);
      x = fma(-CHEM_LDLU(lu + 3032), b[134], x);
      x = fma(-CHEM_LDLU(lu + 3033), b[187], x);
      x = fma(-CHEM_LDLU(lu + 3034), b[188], x);
      b[43] = x * CHEM_LDLU(vd + 43);
    }
    {
      double x = b[42];
      x = fma(-CHEM_LDLU(lu + 3035), b[134], x);
      x = fma(-CHEM_LDLU(lu + 3036), b[187], x);
      x = fma(-CHEM_LDLU(lu + 3037), b[188], x);
      b[42] = x * CHEM_LDLU(vd + 42);
    }
    {
      double x = b[41];
      x = fma(-CHEM_LDLU(lu + 3038), b[162], x);
      x = fma(-CHEM_LDLU(lu + 3039), b[186], x);
      x = fma(-CHEM_LDLU(lu + 3040), b[188], x);
      b[41] = x * CHEM_LDLU(vd + 41);
    }
    {
      double x = b[40];
      x = fma(-CHEM_LDLU(lu + 3041), b[185], x);
      x = fma(-CHEM_LDLU(lu + 3042), b[187], x);
      x = fma(-CHEM_LDLU(lu + 3043), b[188], x);
      b[40] = x * CHEM_LDLU(vd + 40);
    }
    {
      double x = b[39];
      x = fma(-CHEM_LDLU(lu + 3044), b[86], x);
      x = fma(-CHEM_LDLU(lu + 3045), b[162], x);
      x = fma(-CHEM_LDLU(lu + 3046), b[186], x);
      x = fma(-CHEM_LDLU(lu + 3047), b[188], x);
      b[39] = x * CHEM_LDLU(vd + 39);
    }
    {
      double x = b[38];
      x = fma(-CHEM_LDLU(lu + 3048), b[86], x);
      x = fma(-CHEM_LDLU(lu + 3049), b[162], x);
      x = fma(-CHEM_LDLU(lu + 3050), b[188], x);
      b[38] = x * CHEM_LDLU(vd + 38);
    }
    {
      double x = b[37];
      x = fma(-CHEM_LDLU(lu + 3051), b[182], x);
      x = fma(-CHEM_LDLU(lu + 3052), b[185], x);
      x = fma(-CHEM_LDLU(lu + 3053), b[188], x);
      b[37] = x * CHEM_LDLU(vd + 37);
    }
    {
      double x = b[36];
      x = fma(-CHEM_LDLU(lu + 3054), b[162], x);
      x = fma(-CHEM_LDLU(lu + 3055), b[186], x);
      x = fma(-CHEM_LDLU(lu + 3056), b[188], x);
      b[36] = x * CHEM_LDLU(vd + 36);
    }
    {
      double x = b[35];
      x = fma(-CHEM_LDLU(lu + 3057), b[86], x);
      x = fma(-CHEM_LDLU(lu + 3058), b[162], x);
      x = fma(-CHEM_LDLU(lu + 3059), b[188], x);
      b[35] = x * CHEM_LDLU(vd + 35);
    }
    {
      double x = b[34];
      x = fma(-CHEM_LDLU(lu + 3060), b[181], x);
      x = fma(-CHEM_LDLU(lu + 3061), b[185], x);
      x = fma(-CHEM_LDLU(lu + 3062), b[188], x);
      b[34] = x * CHEM_LDLU(vd + 34);
    }
    {
      double x = b[33];
      x = fma(-CHEM_LDLU(lu + 3063), b[43], x);
      b[33] = x * CHEM_LDLU(vd + 33);
    }
    {
      double x = b[32];
      x = fma(-CHEM_LDLU(lu + 3064), b[185], x);
      x = fma(-CHEM_LDLU(lu + 3065), b[186], x);
      b[32] = x * CHEM_LDLU(vd + 32);
    }
    {
      double x = b[31];
      x = fma(-CHEM_LDLU(lu + 3066), b[188], x);
      b[31] = x * CHEM_LDLU(vd + 31);
    }
    {
      double x = b[30];
      b[30] = x * CHEM_LDLU(vd + 30);
    }
    {
      double x = b[29];
      x = fma(-CHEM_LDLU(lu + 3067), b[188], x);
      b[29] = x * CHEM_LDLU(vd + 29);
    }
    {
      double x = b[28];
      x = fma(-CHEM_LDLU(lu + 3068), b[188], x);
      b[28] = x * CHEM_LDLU(vd + 28);
    }
    {
      double x = b[27];
      x = fma(-CHEM_LDLU(lu + 3069), b[188], x);
      b[27] = x * CHEM_LDLU(vd + 27);
    }
    {
      double x = b[26];
      x = fma(-CHEM_LDLU(lu + 3070), b[188], x);
      b[26] = x * CHEM_LDLU(vd + 26);
    }
    {
      double x = b[25];
      x = fma(-CHEM_LDLU(lu + 3071), b[188], x);
      b[25] = x * CHEM_LDLU(vd + 25);
    }
    {
      double x = b[24];
      x = fma(-CHEM_LDLU(lu + 3072), b[188], x);
      b[24] = x * CHEM_LDLU(vd + 24);
    }
    {
      double x = b[23];
      x = fma(-CHEM_LDLU(lu + 3073), b[188], x);
      b[23] = x * CHEM_LDLU(vd + 23);
    }
    {
      double x = b[22];
      x = fma(-CHEM_LDLU(lu + 3074), b[188], x);
      b[22] = x * CHEM_LDLU(vd + 22);
    }
    {
      double x = b[21];
      x = fma(-CHEM_LDLU(lu + 3075), b[188], x);
      b[21] = x * CHEM_LDLU(vd + 21);
    }
    {
      double x = b[20];
      x = fma(-CHEM_LDLU(lu + 3076), b[188], x);
      b[20] = x * CHEM_LDLU(vd + 20);
    }
    {
      double x = b[19];
      x = fma(-CHEM_LDLU(lu + 3077), b[188], x);
      b[19] = x * CHEM_LDLU(vd + 19);
    }
    {
      double x = b[18];
      x = fma(-CHEM_LDLU(lu + 3078), b[162], x);
      b[18] = x * CHEM_LDLU(vd + 18);
    }
    {
      double x = b[17];
      x = fma(-CHEM_LDLU(lu + 3079), b[33], x);
      b[17] = x * CHEM_LDLU(vd + 17);
    }
    {
      double x = b[16];
      x = fma(-CHEM_LDLU(lu + 3080), b[33], x);
      b[16] = x * CHEM_LDLU(vd + 16);
    }
    {
      double x = b[15];
      x = fma(-CHEM_LDLU(lu + 3081), b[164], x);
      x = fma(-CHEM_LDLU(lu + 3082), b[168], x);
      b[15] = x * CHEM_LDLU(vd + 15);
    }
    {
      double x = b[14];
      x = fma(-CHEM_LDLU(lu + 3083), b[188], x);
      b[14] = x * CHEM_LDLU(vd + 14);
    }
    {
      double x = b[13];
      x = fma(-CHEM_LDLU(lu + 3084), b[188], x);
      b[13] = x * CHEM_LDLU(vd + 13);
    }
    {
      double x = b[12];
      x = fma(-CHEM_LDLU(lu + 3085), b[188], x);
      b[12] = x * CHEM_LDLU(vd + 12);
    }
    {
      double x = b[11];
      x = fma(-CHEM_LDLU(lu + 3086), b[188], x);
      b[11] = x * CHEM_LDLU(vd + 11);
    }
    {
      double x = b[10];
      x = fma(-CHEM_LDLU(lu + 3087), b[188], x);
      b[10] = x * CHEM_LDLU(vd + 10);
    }
    {
      double x = b[9];
      x = fma(-CHEM_LDLU(lu + 3088), b[188], x);
      b[9] = x * CHEM_LDLU(vd + 9);
    }
    {
      double x = b[8];
      x = fma(-CHEM_LDLU(lu + 3089), b[188], x);
      b[8] = x * CHEM_LDLU(vd + 8);
    }
    {
      double x = b[7];
      x = fma(-CHEM_LDLU(lu + 3090), b[188], x);
      b[7] = x * CHEM_LDLU(vd + 7);
    }
    {
      double x = b[6];
      x = fma(-CHEM_LDLU(lu + 3091), b[188], x);
      b[6] = x * CHEM_LDLU(vd + 6);
    }
    {
      double x = b[5];
      x = fma(-CHEM_LDLU(lu + 3092), b[188], x);
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
      x = fma(-CHEM_LDLU(lu + 3093), b[69], x);
      b[2] = x * CHEM_LDLU(vd + 2);
    }
    {
      double x = b[1];
      x = fma(-CHEM_LDLU(lu + 3094), b[52], x);
      b[1] = x * CHEM_LDLU(vd + 1);
    }
    {
      double x = b[0];
      x = fma(-CHEM_LDLU(lu + 3095), b[33], x);
      b[0] = x * CHEM_LDLU(vd + 0);
    }
}
}  // namespace mech_cracmm2
