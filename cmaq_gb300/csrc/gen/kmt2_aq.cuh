// Generated by cmaq_gb300/mechgen/kpp_aq.py from CCTM/src/cloud/acm_ae7_kmt2: Henry's law
// constants (aqchem_kmt.F90:371-396), rate constants (aqchem_Initialize.F90:491-636,
// aqchem_Rates.F90:456-579), tolerances, Fun, Jac_SP, KppDecomp, KppSolve as straight-line
// code.  Included inside namespace kmt2 by csrc/kmt2.cuh.  Do not edit.
#pragma once

KQ_HD inline void kq_henry(Cell& c, float t2)
{
    c.henry[0] = (double)kq_hlconst((float)0x1.6666660000000p+0, (float)0x1.6a80000000000p+11, t2);   // SO2H
    c.henry[1] = (double)kq_hlconst((float)0x1.9a28000000000p+17, (float)0x1.0fe0000000000p+13, t2);   // HNO3H
    c.henry[2] = (double)kq_hlconst((float)0x1.26e9780000000p-5, (float)0x1.1300000000000p+11, t2);   // CO2H
    c.henry[3] = (double)kq_hlconst((float)0x1.e800000000000p+5, (float)0x1.0680000000000p+12, t2);   // NH3H
    c.henry[4] = (double)kq_hlconst((float)0x1.adb0000000000p+16, (float)0x1.ce80000000000p+12, t2);   // H2O2H
    c.henry[5] = (double)kq_hlconst((float)0x1.758e220000000p-7, (float)0x1.1f80000000000p+11, t2);   // O3H
    c.henry[6] = (double)kq_hlconst((float)0x1.1620000000000p+13, (float)0x1.7d40000000000p+12, t2);   // FOAH
    c.henry[7] = (double)kq_hlconst((float)0x1.3600000000000p+8, (float)0x1.4500000000000p+12, t2);   // MHPH
    c.henry[8] = (double)kq_hlconst((float)0x1.a400000000000p+9, (float)0x1.4b40000000000p+12, t2);   // PAAH
    c.henry[9] = (double)kq_hlconst((float)0x1.3000000000000p+4, (float)0x1.2c00000000000p+9, t2);   // HCLH
    c.henry[10] = (double)kq_hlconst((float)0x1.5f90000000000p+18, (float)0x0.0p+0, t2);   // GLYH
    c.henry[11] = (double)kq_hlconst((float)0x1.f400000000000p+14, (float)0x0.0p+0, t2);   // MGLYH
    c.henry[12] = (double)kq_hlconst((float)0x1.f400000000000p+11, (float)0x1.70c0000000000p+12, t2);   // HO2H
    c.henry[13] = (double)kq_hlconst((float)0x1.89374c0000000p-7, (float)0x1.3880000000000p+11, t2);   // NO2H
    c.henry[14] = (double)kq_hlconst((float)0x1.9000000000000p+5, (float)0x1.3240000000000p+12, t2);   // HONOH
    c.henry[15] = (double)kq_hlconst((float)0x1.7700000000000p+13, (float)0x1.af40000000000p+12, t2);   // HNO4H
    c.henry[16] = (double)kq_hlconst((float)0x1.e000000000000p+4, (float)0x1.1940000000000p+12, t2);   // HOH
    c.henry[17] = (double)kq_hlconst((float)0x1.c9c3800000000p+24, (float)0x0.0p+0, t2);   // HIEPOX
    c.henry[18] = (double)kq_hlconst((float)0x1.d4c0000000000p+16, (float)0x0.0p+0, t2);   // HMAE
    c.henry[19] = (double)kq_hlconst((float)0x1.d4c0000000000p+16, (float)0x0.0p+0, t2);   // HHMML
    c.henry[20] = 0x1.4050000000000p+15 * kq_exp(0x1.1f80000000000p+12 * ((298.0 - (double)t2) / (298.0 * (double)t2)));   // GCOLH
    c.henry[21] = (double)kq_hlconst((float)0x1.0040000000000p+12, (float)0x1.89c0000000000p+12, t2);   // CCOOHH
    c.henry[22] = 0x1.4000000000000p+1;   // HCHOH
    c.henry[23] = (double)kq_hlconst((float)0x1.24f8000000000p+18, (float)0x1.4500000000000p+12, t2);   // PYRACH
    c.henry[24] = (double)kq_hlconst((float)0x1.3333340000000p-1, (float)0x0.0p+0, t2);   // NO3H
    c.henry[25] = 0x1.599999999999ap+1 * kq_exp(0x1.fb80000000000p+10 * ((298.0 - (double)t2) / (298.0 * (double)t2)));   // CH3O2H
}

KQ_HD KQ_NOINLINE void kq_rates_once(const Cell& c, const double* v, const double* f, double* r, long long s)
{
    (void)v;
    (void)f;
    r[0 * s] = kq_kmtf(c, 0x1.c28f5c28f5c29p-4, 0x1.ad7f29abcaf48p-17, 0x1.004189374bc6ap+6);
    r[1 * s] = kq_kmtf(c, 0x1.63886594af4f1p-4, 0x1.baeb22f9294c3p-17, 0x1.f81a9fbe76c8bp+5);
    r[2 * s] = kq_kmtf(c, 0x1.3a92a30553261p-13, 0x1.040bfe3b03e21p-16, 0x1.60147ae147ae1p+5);
    r[3 * s] = kq_kmtf(c, 0x1.74bc6a7ef9db2p-4, 0x1.81e03f705857bp-16, 0x1.107ef9db22d0ep+4);
    r[4 * s] = kq_kmtf(c, 0x1.39c0ebedfa440p-3, 0x1.e9e50b87f37efp-17, 0x1.101eb851eb852p+5);
    r[5 * s] = kq_kmtf(c, 0x1.999999999999ap-4, 0x1.f09b082ea2aacp-17, 0x1.7ffbe76c8b439p+5);
    r[6 * s] = kq_kmtf(c, 0x1.77318fc504817p-6, 0x1.00b0ffe7ac4c2p-16, 0x1.7033333333333p+5);
    r[7 * s] = kq_kmtf(c, 0x1.bae46cfc829d0p-8, 0x1.b79024a5d1b64p-17, 0x1.8051eb851eb85p+5);
    r[8 * s] = kq_kmtf(c, 0x1.374bc6a7ef9dbp-6, 0x1.56415534e5baep-17, 0x1.3033333333333p+6);
    r[9 * s] = kq_kmtf(c, 0x1.da5119ce075f7p-4, 0x1.3d16e1c3d4d68p-16, 0x1.23b020c49ba5ep+5);
    r[10 * s] = kq_kmtf(c, 0x1.78d4fdf3b645ap-6, 0x1.81e03f705857bp-17, 0x1.d051eb851eb85p+5);
    r[11 * s] = kq_kmtf(c, 0x1.78d4fdf3b645ap-6, 0x1.81e03f705857bp-17, 0x1.203d70a3d70a4p+6);
    r[12 * s] = kq_kmtf(c, 0x1.47ae147ae147bp-7, 0x1.5cf751db94e6bp-17, 0x1.08147ae147ae1p+5);
    r[13 * s] = kq_kmtf(c, 0x1.89374bc6a7efap-10, 0x1.421f5f40d8376p-16, 0x1.70147ae147ae1p+5);
    r[14 * s] = kq_kmtf(c, 0x1.0000000000000p-1, 0x1.b43526527a205p-17, 0x1.78147ae147ae1p+5);
    r[15 * s] = kq_kmtf(c, 0x1.999999999999ap-4, 0x1.b43526527a205p-17, 0x1.3c0a3d70a3d71p+6);
    r[16 * s] = kq_kmtb(c, c.henry[0], 0x1.c28f5c28f5c29p-4, 0x1.ad7f29abcaf48p-17, 0x1.004189374bc6ap+6);
    r[17 * s] = kq_kmtb(c, c.henry[1], 0x1.63886594af4f1p-4, 0x1.baeb22f9294c3p-17, 0x1.f81a9fbe76c8bp+5);
    r[18 * s] = kq_kmtb(c, c.henry[2], 0x1.3a92a30553261p-13, 0x1.040bfe3b03e21p-16, 0x1.60147ae147ae1p+5);
    r[19 * s] = kq_kmtb(c, c.henry[3], 0x1.74bc6a7ef9db2p-4, 0x1.81e03f705857bp-16, 0x1.107ef9db22d0ep+4);
    r[20 * s] = kq_kmtb(c, c.henry[4], 0x1.39c0ebedfa440p-3, 0x1.e9e50b87f37efp-17, 0x1.101eb851eb852p+5);
    r[21 * s] = kq_kmtb(c, c.henry[5], 0x1.999999999999ap-4, 0x1.f09b082ea2aacp-17, 0x1.7ffbe76c8b439p+5);
    r[22 * s] = kq_kmtb(c, c.henry[6], 0x1.77318fc504817p-6, 0x1.00b0ffe7ac4c2p-16, 0x1.7033333333333p+5);
    r[23 * s] = kq_kmtb(c, c.henry[7], 0x1.bae46cfc829d0p-8, 0x1.b79024a5d1b64p-17, 0x1.8051eb851eb85p+5);
    r[24 * s] = kq_kmtb(c, c.henry[8], 0x1.374bc6a7ef9dbp-6, 0x1.56415534e5baep-17, 0x1.3033333333333p+6);
    r[25 * s] = kq_kmtb(c, c.henry[9], 0x1.da5119ce075f7p-4, 0x1.3d16e1c3d4d68p-16, 0x1.23b020c49ba5ep+5);
    r[26 * s] = kq_kmtb(c, c.henry[10], 0x1.78d4fdf3b645ap-6, 0x1.81e03f705857bp-17, 0x1.d051eb851eb85p+5);
    r[27 * s] = kq_kmtb(c, c.henry[11], 0x1.78d4fdf3b645ap-6, 0x1.81e03f705857bp-17, 0x1.203d70a3d70a4p+6);
    r[28 * s] = kq_kmtb(c, c.henry[12], 0x1.47ae147ae147bp-7, 0x1.5cf751db94e6bp-17, 0x1.08147ae147ae1p+5);
    r[29 * s] = kq_kmtb(c, c.henry[13], 0x1.89374bc6a7efap-10, 0x1.421f5f40d8376p-16, 0x1.70147ae147ae1p+5);
    r[30 * s] = kq_kmtb(c, c.henry[14], 0x1.0000000000000p-1, 0x1.b43526527a205p-17, 0x1.78147ae147ae1p+5);
    r[31 * s] = kq_kmtb(c, c.henry[15], 0x1.999999999999ap-4, 0x1.b43526527a205p-17, 0x1.3c0a3d70a3d71p+6);
    r[32 * s] = c.alfa3;
    r[33 * s] = c.alfa3;
    r[34 * s] = c.alfa3;
    r[35 * s] = c.alfa3;
    r[36 * s] = c.alfa3;
    r[37 * s] = c.alfa3;
    r[38 * s] = c.alfa3;
    r[39 * s] = c.alfa3;
    r[91 * s] = 0x1.199999999999ap+0;
    r[95 * s] = c.wetfac;
    r[96 * s] = c.wetfac;
    r[97 * s] = c.wetfac;
    r[98 * s] = c.wetfac;
    r[99 * s] = c.wetfac;
    r[100 * s] = c.wetfac;
    r[101 * s] = c.wetfac;
    r[102 * s] = c.wetfac;
    r[103 * s] = c.wetfac;
    r[104 * s] = c.wetfac;
    r[105 * s] = c.wetfac;
    r[106 * s] = c.wetfac;
    r[107 * s] = c.wetfac;
    r[108 * s] = c.wetfac;
    r[109 * s] = c.wetfac;
    r[110 * s] = c.wetfac;
    r[111 * s] = c.wetfac;
    r[112 * s] = c.wetfac;
    r[113 * s] = c.wetfac;
    r[114 * s] = c.wetfac;
    r[115 * s] = c.wetfac;
    r[116 * s] = c.wetfac;
    r[117 * s] = c.wetfac;
    r[118 * s] = c.wetfac;
    r[119 * s] = c.wetfac;
    r[120 * s] = c.wetfac;
    r[121 * s] = c.wetfac;
    r[122 * s] = c.wetfac;
    r[123 * s] = c.wetfac;
    r[124 * s] = c.wetfac;
    r[125 * s] = c.wetfac;
    r[126 * s] = c.wetfac;
    r[127 * s] = c.wetfac;
    r[128 * s] = c.wetfac;
    r[129 * s] = c.wetfac;
    r[130 * s] = c.wetfac;
    r[131 * s] = c.wetfac;
    r[132 * s] = c.wetfac;
    r[133 * s] = c.wetfac;
    r[134 * s] = c.wetfac;
    r[135 * s] = c.wetfac;
    r[136 * s] = c.wetfac;
    r[137 * s] = kq_kmtf(c, 0x1.999999999999ap-5, 0x1.00b0ffe7ac4c2p-16, 0x1.101cac083126fp+4);
    r[138 * s] = kq_kmtb(c, c.henry[16], 0x1.999999999999ap-5, 0x1.00b0ffe7ac4c2p-16, 0x1.101cac083126fp+4);
    r[139 * s] = c.wetfac;
    r[140 * s] = kq_kmtf(c, 0x1.47ae147ae147bp-6, 0x1.4f8b588e368f1p-17, 0x1.d8851eb851eb8p+6);
    r[141 * s] = kq_kmtf(c, 0x1.47ae147ae147bp-6, 0x1.4f8b588e368f1p-17, 0x1.9800000000000p+6);
    r[142 * s] = kq_kmtf(c, 0x1.47ae147ae147bp-6, 0x1.4f8b588e368f1p-17, 0x1.9800000000000p+6);
    r[143 * s] = kq_kmtb(c, c.henry[17], 0x1.47ae147ae147bp-6, 0x1.4f8b588e368f1p-17, 0x1.d8851eb851eb8p+6);
    r[144 * s] = kq_kmtb(c, c.henry[18], 0x1.47ae147ae147bp-6, 0x1.4f8b588e368f1p-17, 0x1.9800000000000p+6);
    r[145 * s] = kq_kmtb(c, c.henry[19], 0x1.47ae147ae147bp-6, 0x1.4f8b588e368f1p-17, 0x1.9800000000000p+6);
    r[157 * s] = c.wetfac;
    r[158 * s] = c.wetfac;
    r[159 * s] = c.wetfac;
    r[160 * s] = c.wetfac;
    r[161 * s] = c.wetfac;
    r[162 * s] = c.wetfac;
    r[163 * s] = c.wetfac;
    r[164 * s] = c.wetfac;
    r[165 * s] = c.wetfac;
    r[166 * s] = kq_kmtf(c, 0x1.78d4fdf3b645ap-6, 0x1.81e03f705857bp-17, 0x1.e06a7ef9db22dp+5);
    r[167 * s] = kq_kmtf(c, 0x1.07c84b5dcc63fp-5, 0x1.a013305e6c9cep-17, 0x1.e06a7ef9db22dp+5);
    r[168 * s] = kq_kmtf(c, 0x1.47ae147ae147bp-6, 0x1.132576b20e04ap-16, 0x1.e07ae147ae148p+4);
    r[169 * s] = kq_kmtf(c, 0x1.47ae147ae147bp-6, 0x1.132576b20e04ap-16, 0x1.e07ae147ae148p+4);
    r[170 * s] = (double)c.mtpyrac * kq_kmtf(c, 0x1.07c84b5dcc63fp-5, 0x1.a013305e6c9cep-17, 0x1.603d70a3d70a4p+6);
    r[171 * s] = kq_kmtb(c, c.henry[20], 0x1.78d4fdf3b645ap-6, 0x1.81e03f705857bp-17, 0x1.e06a7ef9db22dp+5);
    r[172 * s] = kq_kmtb(c, c.henry[21], 0x1.07c84b5dcc63fp-5, 0x1.a013305e6c9cep-17, 0x1.e06a7ef9db22dp+5);
    r[173 * s] = kq_kmtb(c, c.henry[22], 0x1.47ae147ae147bp-6, 0x1.132576b20e04ap-16, 0x1.e07ae147ae148p+4);
    r[174 * s] = kq_kmtb(c, c.henry[22], 0x1.47ae147ae147bp-6, 0x1.132576b20e04ap-16, 0x1.e07ae147ae148p+4);
    r[175 * s] = (double)c.mtpyrac * kq_kmtb(c, c.henry[23], 0x1.07c84b5dcc63fp-5, 0x1.a013305e6c9cep-17, 0x1.603d70a3d70a4p+6);
    r[188 * s] = kq_hydf(c, 0x1.70a3d70a3d70ap-3, 0x1.f7c0000000000p+11);
    r[189 * s] = 0x1.4e3bcd35a8588p-8;
    r[190 * s] = kq_hydf(c, 0x1.70a3d70a3d70ap-3, 0x1.f7c0000000000p+11);
    r[191 * s] = 0x1.4e3bcd35a8588p-8;
    r[192 * s] = kq_kphot(c, 0x1.34b365f379dfcp-18, c.jh2o2);
    r[211 * s] = c.wetfac;
    r[212 * s] = c.wetfac;
    r[213 * s] = c.wetfac;
    r[214 * s] = c.wetfac;
    r[215 * s] = c.wetfac;
    r[216 * s] = c.wetfac;
    r[217 * s] = c.wetfac;
    r[218 * s] = c.wetfac;
    r[219 * s] = c.wetfac;
    r[220 * s] = c.wetfac;
    r[221 * s] = c.wetfac;
    r[222 * s] = c.wetfac;
    r[223 * s] = c.wetfac;
    r[224 * s] = c.wetfac;
    r[225 * s] = c.wetfac;
    r[226 * s] = c.wetfac;
    r[227 * s] = kq_kmtf(c, 0x1.999999999999ap-5, 0x1.4f8b588e368f1p-17, 0x1.f000000000000p+5);
    r[228 * s] = kq_kmtf(c, 0x1.999999999999ap-5, 0x1.c4fc1df3300dep-17, 0x1.8800000000000p+5);
    r[229 * s] = kq_kmtb(c, c.henry[24], 0x1.999999999999ap-5, 0x1.4f8b588e368f1p-17, 0x1.f000000000000p+5);
    r[230 * s] = kq_kmtb(c, c.henry[25], 0x1.999999999999ap-5, 0x1.c4fc1df3300dep-17, 0x1.8800000000000p+5);
    r[231 * s] = kq_kphot(c, 0x1.2ca5d05ea7ab3p-21, -0x1.0000000000000p+0);
    r[260 * s] = c.wetfac;
    r[261 * s] = c.wetfac;
    r[262 * s] = c.wetfac;
    r[263 * s] = c.wetfac;
    r[264 * s] = c.wetfac;
    r[265 * s] = c.wetfac;
    r[266 * s] = c.wetfac;
    r[267 * s] = c.wetfac;
    r[268 * s] = c.wetfac;
}

KQ_HD KQ_NOINLINE void kq_rates_update(const Cell& c, const double* v, const double* f, double* r, long long s)
{
    r[40 * s] = kq_disf(c, 0x1.c779a6b50b0f2p-7, 0x1.d380000000000p+10, 0x1.7d78400000000p+27, 0);
    r[41 * s] = kq_disf(c, 0x1.209f2e6f59483p-24, 0x1.6300000000000p+8, 0x1.74876e8000000p+35, 1);
    r[42 * s] = kq_disf(c, 0x1.1000000000000p+4, 0x0.0p+0, 0x1.74876e8000000p+35, 0);
    r[43 * s] = kq_disf(c, 0x1.cdb57fff13c6ep-22, -0x1.f180000000000p+9, 0x1.f400000000000p+15, 0);
    r[44 * s] = kq_disf(c, 0x1.9ba83b3532653p-35, -0x1.be40000000000p+10, 0x1.74876e8000000p+35, 1);
    r[45 * s] = kq_disf(c, 0x1.28f4ebcfc7531p-16, -0x1.6300000000000p+9, 0x1.faa3b50000000p+34, 0);
    r[46 * s] = kq_disf(c, 0x1.797cc39ffd60fp-13, -0x1.4000000000000p+4, 0x1.74876e8000000p+35, 0);
    r[47 * s] = kq_disf(c, 0x1.a8ce000000000p+20, 0x1.aea0000000000p+12, 0x1.74876e8000000p+35, 0);
    r[48 * s] = kq_disf(c, 0x1.9f0d3ef0faf29p-53, -0x1.b2b0000000000p+12, 0x1.04c533c000000p+37, 0);
    r[49 * s] = kq_disf(c, 0x1.f400000000000p+9, 0x0.0p+0, 0x1.74876e8000000p+35, 0);
    r[50 * s] = kq_disf(c, 0x1.4e3bcd35a8588p-7, 0x1.31a0000000000p+11, 0x1.74876e8000000p+36, 1);
    r[51 * s] = kq_disf(c, 0x1.0c6f7a0b5ed8dp-16, 0x0.0p+0, 0x1.74876e8000000p+35, 0);
    r[52 * s] = kq_disf(c, 0x1.15df6555c52e7p-11, -0x1.b800000000000p+10, 0x1.74876e8000000p+35, 0);
    r[53 * s] = kq_disf(c, 0x1.4f8b588e368f1p-17, 0x0.0p+0, 0x1.74876e8000000p+35, 0);
    r[54 * s] = kq_disb(c, 0x1.7d78400000000p+27, 2);
    r[55 * s] = kq_disb(c, 0x1.74876e8000000p+35, 1);
    r[56 * s] = kq_disb(c, 0x1.74876e8000000p+35, 2);
    r[57 * s] = kq_disb(c, 0x1.f400000000000p+15, 2);
    r[58 * s] = kq_disb(c, 0x1.74876e8000000p+35, 1);
    r[59 * s] = kq_disb(c, 0x1.faa3b50000000p+34, 2);
    r[60 * s] = kq_disb(c, 0x1.74876e8000000p+35, 2);
    r[61 * s] = kq_disb(c, 0x1.74876e8000000p+35, 2);
    r[62 * s] = kq_disb(c, 0x1.04c533c000000p+37, 2);
    r[63 * s] = kq_disb(c, 0x1.74876e8000000p+35, 2);
    r[64 * s] = kq_disb(c, 0x1.74876e8000000p+36, 1);
    r[65 * s] = kq_disb(c, 0x1.74876e8000000p+35, 2);
    r[66 * s] = kq_disb(c, 0x1.74876e8000000p+35, 2);
    r[67 * s] = kq_disb(c, 0x1.74876e8000000p+35, 2);
    r[68 * s] = kq_krxn(c, v, s, 0x1.1c31e80000000p+26, -0x1.294147ae147aep+12, 1, 0, 0);
    r[69 * s] = kq_krxn(c, v, s, 0x1.7700000000000p+14, 0x0.0p+0, 0, 1, 0);
    r[70 * s] = kq_krxn(c, v, s, 0x1.6954000000000p+18, -0x1.59ae147ae147bp+12, 0, 2, 0);
    r[71 * s] = kq_krxn(c, v, s, 0x1.65a0bc0000000p+30, -0x1.4a08f5c28f5c3p+12, 0, 3, 0);
    r[72 * s] = kq_krxn(c, v, s, 0x1.7700000000000p+9, 0x0.0p+0, 0, 0, 1);
    r[73 * s] = kq_krxn(c, v, s, 0x1.7700000000000p+9, 0x0.0p+0, 0, 0, 1);
    r[74 * s] = kq_krxn(c, v, s, 0x1.7700000000000p+9, 0x0.0p+0, 0, 0, 1);
    r[75 * s] = kq_krxn(c, v, s, 0x1.4500000000000p+11, 0x0.0p+0, 0, 0, 1);
    r[76 * s] = kq_krxn(c, v, s, 0x1.4500000000000p+11, 0x0.0p+0, 0, 0, 1);
    r[77 * s] = kq_krxn(c, v, s, 0x1.4500000000000p+11, 0x0.0p+0, 0, 0, 1);
    r[78 * s] = kq_krxn(c, v, s, 0x1.2a05f20000000p+33, 0x0.0p+0, 3, 0, 1);
    r[79 * s] = kq_krxn(c, v, s, 0x1.2a05f20000000p+33, 0x0.0p+0, 3, 0, 1);
    r[80 * s] = kq_krxn(c, v, s, 0x1.2a05f20000000p+33, 0x0.0p+0, 3, 0, 1);
    r[81 * s] = kq_krxn(c, v, s, 0x1.21eac00000000p+24, -0x1.daf0000000000p+11, 3, 0, 0);
    r[82 * s] = kq_krxn(c, v, s, 0x1.12a8800000000p+25, -0x1.f3e6666666666p+11, 3, 0, 0);
    r[83 * s] = kq_krxn(c, v, s, 0x1.5e00000000000p+9, 0x0.0p+0, 0, 0, 0);
    r[84 * s] = kq_krxn(c, v, s, 0x1.9546000000000p+19, -0x1.5180000000000p+11, 0, 0, 0);
    r[85 * s] = kq_krxn(c, v, s, 0x1.6e36000000000p+26, -0x1.c700000000000p+9, 0, 0, 0);
    r[86 * s] = kq_krxn(c, v, s, 0x1.65a0bc0000000p+30, -0x1.7700000000000p+10, 0, 0, 0);
    r[87 * s] = kq_krxn(c, v, s, 0x1.e848000000000p+20, 0x0.0p+0, 0, 0, 0);
    r[88 * s] = kq_krxn(c, v, s, 0x1.e848000000000p+20, 0x0.0p+0, 0, 0, 0);
    r[89 * s] = kq_krxn(c, v, s, 0x1.e848000000000p+20, 0x0.0p+0, 0, 0, 0);
    r[90 * s] = kq_krxn(c, v, s, 0x1.4244000000000p+18, 0x0.0p+0, 0, 0, 0);
    r[92 * s] = kq_krxn(c, v, s, 0x1.e848000000000p+18, -0x1.b580000000000p+12, 0, 0, 0);
    r[93 * s] = kq_krxn(c, v, s, 0x1.2a05f20000000p+33, 0x0.0p+0, 0, 0, 0);
    r[94 * s] = kq_krxn(c, v, s, 0x1.2a05f20000000p+33, 0x0.0p+0, 0, 0, 0);
    r[146 * s] = kq_kiepox(c, v, f, s, 0x1.d7dbf487fcb92p-11, 0x1.b79024a5d1b64p-17, 1);
    r[147 * s] = kq_kiepox(c, v, f, s, 0x1.2157689ca18bdp-7, 0x1.87ea6f9ff5ff2p-19, 1);
    r[148 * s] = kq_kiepox(c, v, f, s, 0x1.a36e2eb1c432dp-13, 0x1.87ea6f9ff5ff2p-19, 1);
    r[149 * s] = kq_kiepox(c, v, f, s, 0x1.a36e2eb1c432dp-13, 0x1.87ea6f9ff5ff2p-19, 1);
    r[150 * s] = kq_kiepox(c, v, f, s, 0x1.d7dbf487fcb92p-11, 0x1.b79024a5d1b64p-17, 0);
    r[151 * s] = kq_kiepox(c, v, f, s, 0x1.2157689ca18bdp-7, 0x1.87ea6f9ff5ff2p-19, 0);
    r[152 * s] = kq_kiepox(c, v, f, s, 0x1.a36e2eb1c432dp-13, 0x1.87ea6f9ff5ff2p-19, 0);
    r[153 * s] = kq_kiepox(c, v, f, s, 0x1.d7dbf487fcb92p-11, 0x1.b79024a5d1b64p-17, 2);
    r[154 * s] = kq_kiepox(c, v, f, s, 0x1.a36e2eb1c432dp-13, 0x1.87ea6f9ff5ff2p-19, 2);
    r[155 * s] = kq_kiepox(c, v, f, s, 0x1.d7dbf487fcb92p-11, 0x1.b79024a5d1b64p-17, 2);
    r[156 * s] = kq_kiepox(c, v, f, s, 0x1.a36e2eb1c432dp-13, 0x1.87ea6f9ff5ff2p-19, 2);
    r[176 * s] = kq_disf(c, 0x1.6bdb1a6d698fep-12, -0x1.0b00000000000p+8, 0x1.2a05f20000000p+34, 0);
    r[177 * s] = kq_disf(c, 0x1.cac083126e979p-5, -0x1.c500000000000p+8, 0x1.74876e8000000p+35, 0);
    r[178 * s] = kq_disf(c, 0x1.c6a99d1cdbd8ep-15, -0x1.9280000000000p+9, 0x1.74876e8000000p+35, 1);
    r[179 * s] = kq_disf(c, 0x1.a36e2eb1c432dp-9, 0x0.0p+0, 0x1.2a05f20000000p+34, 0);
    r[180 * s] = kq_disf(c, 0x1.3660e51d25aabp-13, -0x1.4200000000000p+6, 0x1.2a05f20000000p+34, 0);
    r[181 * s] = kq_disf(c, 0x1.2599ed7c6fbd2p-16, 0x1.7000000000000p+5, 0x1.74876e8000000p+35, 0);
    r[182 * s] = kq_disb(c, 0x1.2a05f20000000p+34, 2);
    r[183 * s] = kq_disb(c, 0x1.74876e8000000p+35, 2);
    r[184 * s] = kq_disb(c, 0x1.74876e8000000p+35, 1);
    r[185 * s] = kq_disb(c, 0x1.2a05f20000000p+34, 2);
    r[186 * s] = kq_disb(c, 0x1.2a05f20000000p+34, 2);
    r[187 * s] = kq_disb(c, 0x1.74876e8000000p+35, 2);
    r[193 * s] = kq_krxn(c, v, s, 0x1.dcd6500000000p+28, 0x0.0p+0, 0, 0, 0);
    r[194 * s] = kq_krxn(c, v, s, 0x1.dcd6500000000p+29, 0x0.0p+0, 0, 0, 0);
    r[195 * s] = kq_krxn(c, v, s, 0x1.1e1a300000000p+29, 0x0.0p+0, 0, 0, 0);
    r[196 * s] = kq_krxn(c, v, s, 0x1.9a14780000000p+29, 0x0.0p+0, 0, 0, 0);
    r[197 * s] = kq_krxn(c, v, s, 0x1.0642ac0000000p+30, -0x1.7b00000000000p+10, 0, 0, 0);
    r[198 * s] = kq_krxn(c, v, s, 0x1.1e1a300000000p+27, 0x0.0p+0, 0, 0, 0);
    r[199 * s] = kq_krxn(c, v, s, 0x1.1e1a300000000p+30, 0x0.0p+0, 0, 0, 0);
    r[200 * s] = kq_krxn(c, v, s, 0x1.55cc000000000p+20, 0x0.0p+0, 0, 0, 0);
    r[201 * s] = kq_krxn(c, v, s, 0x1.6694e00000000p+25, 0x0.0p+0, 0, 0, 0);
    r[202 * s] = kq_krxn(c, v, s, 0x1.d5f8800000000p+22, 0x0.0p+0, 0, 0, 0);
    r[203 * s] = kq_krxn(c, v, s, 0x1.4dc9380000000p+29, 0x0.0p+0, 0, 0, 0);
    r[204 * s] = kq_krxn(c, v, s, 0x1.c9c3800000000p+25, 0x0.0p+0, 0, 0, 0);
    r[205 * s] = kq_krxn(c, v, s, 0x1.c9c3800000000p+25, 0x0.0p+0, 0, 0, 0);
    r[206 * s] = kq_krxn(c, v, s, 0x1.e848000000000p+23, 0x0.0p+0, 0, 0, 0);
    r[207 * s] = kq_krxn(c, v, s, 0x1.443fd00000000p+26, 0x0.0p+0, 0, 0, 0);
    r[208 * s] = kq_krxn(c, v, s, 0x1.0642ac0000000p+30, -0x1.fe00000000000p+9, 0, 0, 0);
    r[209 * s] = kq_krxn(c, v, s, 0x1.c9c3800000000p+26, -0x1.ef00000000000p+9, 0, 0, 0);
    r[210 * s] = kq_krxn(c, v, s, 0x1.0642ac0000000p+30, -0x1.fe00000000000p+9, 0, 0, 0);
    r[232 * s] = kq_krxn(c, v, s, 0x1.ad27480000000p+31, -0x1.d100000000000p+9, 0, 0, 0);
    r[233 * s] = kq_krxn(c, v, s, 0x1.a13b860000000p+34, 0x0.0p+0, 0, 0, 0);
    r[234 * s] = kq_krxn(c, v, s, 0x1.04c533c000000p+35, -0x1.6800000000000p+9, 0, 0, 0);
    r[235 * s] = kq_krxn(c, v, s, 0x1.e848000000000p+24, -0x1.a900000000000p+10, 0, 0, 0);
    r[236 * s] = kq_krxn(c, v, s, 0x1.41dd760000000p+31, 0x0.0p+0, 0, 0, 0);
    r[237 * s] = kq_krxn(c, v, s, 0x1.ad27480000000p+30, 0x0.0p+0, 0, 0, 0);
    r[238 * s] = kq_krxn(c, v, s, 0x1.0c388d0000000p+32, 0x0.0p+0, 0, 0, 0);
    r[239 * s] = kq_krxn(c, v, s, 0x1.a9fbe76c8b439p-6, 0x0.0p+0, 4, 0, 0);
    r[240 * s] = kq_krxn(c, v, s, 0x1.86a0000000000p+16, 0x0.0p+0, 0, 0, 0);
    r[241 * s] = kq_krxn(c, v, s, 0x1.35f1b40000000p+30, -0x1.1300000000000p+11, 0, 0, 0);
    r[242 * s] = kq_krxn(c, v, s, 0x1.0642ac0000000p+30, 0x0.0p+0, 0, 0, 0);
    r[243 * s] = kq_krxn(c, v, s, 0x1.954fc40000000p+30, 0x0.0p+0, 0, 0, 0);
    r[244 * s] = kq_krxn(c, v, s, 0x1.a39de00000000p+27, -0x1.4500000000000p+11, 0, 0, 0);
    r[245 * s] = kq_krxn(c, v, s, 0x1.b159800000000p+22, 0x0.0p+0, 3, 0, 0);
    r[246 * s] = kq_krxn(c, v, s, 0x1.cc00000000000p+8, -0x1.1300000000000p+10, 0, 0, 0);
    r[247 * s] = kq_krxn(c, v, s, 0x1.443fd00000000p+27, -0x1.1300000000000p+11, 0, 0, 0);
    r[248 * s] = kq_krxn(c, v, s, 0x1.e848000000000p+18, 0x0.0p+0, 0, 0, 0);
    r[249 * s] = kq_krxn(c, v, s, 0x1.954fc40000000p+31, -0x1.2c00000000000p+10, 0, 0, 0);
    r[250 * s] = kq_krxn(c, v, s, 0x1.8b00000000000p+9, -0x1.6a80000000000p+11, 0, 0, 0);
    r[251 * s] = kq_krxn(c, v, s, 0x1.7d78400000000p+24, -0x1.3240000000000p+11, 0, 0, 0);
    r[252 * s] = kq_krxn(c, v, s, 0x1.f8a0902de00d2p-8, -0x1.1f80000000000p+13, 4, 0, 0);
    r[253 * s] = kq_krxn(c, v, s, 0x1.ce80000000000p+11, 0x0.0p+0, 0, 0, 0);
    r[254 * s] = kq_krxn(c, v, s, 0x1.1e1a300000000p+28, 0x0.0p+0, 0, 0, 0);
    r[255 * s] = kq_krxn(c, v, s, 0x1.8b00000000000p+9, -0x1.6a80000000000p+11, 0, 0, 0);
    r[256 * s] = kq_krxn(c, v, s, 0x1.7d78400000000p+24, -0x1.3240000000000p+11, 0, 0, 0);
    r[257 * s] = kq_krxn(c, v, s, 0x1.f8a0902de00d2p-8, -0x1.1f80000000000p+13, 4, 0, 0);
    r[258 * s] = kq_krxn(c, v, s, 0x1.ce80000000000p+11, 0x0.0p+0, 0, 0, 0);
    r[259 * s] = kq_krxn(c, v, s, 0x1.1e1a300000000p+28, 0x0.0p+0, 0, 0, 0);
}

KQ_HD inline double kq_rtol(int i) { return (i == 101 || i == 105 || i == 112 || i == 145) ? 0x1.0624dd2f1a9fcp-10 : 0x1.47ae147ae147bp-7; }
KQ_HD inline double kq_atol(int) { return 0x1.47ae147ae147bp-7; }

KQ_HD inline void kq_add_diagonal(double* g, double x, long long s)
{
    g[0 * s] = g[0 * s] + x;
    g[1 * s] = g[1 * s] + x;
    g[2 * s] = g[2 * s] + x;
    g[3 * s] = g[3 * s] + x;
    g[4 * s] = g[4 * s] + x;
    g[5 * s] = g[5 * s] + x;
    g[6 * s] = g[6 * s] + x;
    g[7 * s] = g[7 * s] + x;
    g[9 * s] = g[9 * s] + x;
    g[11 * s] = g[11 * s] + x;
    g[12 * s] = g[12 * s] + x;
    g[14 * s] = g[14 * s] + x;
    g[15 * s] = g[15 * s] + x;
    g[16 * s] = g[16 * s] + x;
    g[17 * s] = g[17 * s] + x;
    g[18 * s] = g[18 * s] + x;
    g[19 * s] = g[19 * s] + x;
    g[21 * s] = g[21 * s] + x;
    g[22 * s] = g[22 * s] + x;
    g[31 * s] = g[31 * s] + x;
    g[33 * s] = g[33 * s] + x;
    g[38 * s] = g[38 * s] + x;
    g[42 * s] = g[42 * s] + x;
    g[44 * s] = g[44 * s] + x;
    g[46 * s] = g[46 * s] + x;
    g[48 * s] = g[48 * s] + x;
    g[51 * s] = g[51 * s] + x;
    g[53 * s] = g[53 * s] + x;
    g[55 * s] = g[55 * s] + x;
    g[59 * s] = g[59 * s] + x;
    g[61 * s] = g[61 * s] + x;
    g[63 * s] = g[63 * s] + x;
    g[65 * s] = g[65 * s] + x;
    g[67 * s] = g[67 * s] + x;
    g[69 * s] = g[69 * s] + x;
    g[71 * s] = g[71 * s] + x;
    g[74 * s] = g[74 * s] + x;
    g[76 * s] = g[76 * s] + x;
    g[78 * s] = g[78 * s] + x;
    g[80 * s] = g[80 * s] + x;
    g[82 * s] = g[82 * s] + x;
    g[84 * s] = g[84 * s] + x;
    g[85 * s] = g[85 * s] + x;
    g[88 * s] = g[88 * s] + x;
    g[90 * s] = g[90 * s] + x;
    g[92 * s] = g[92 * s] + x;
    g[94 * s] = g[94 * s] + x;
    g[95 * s] = g[95 * s] + x;
    g[97 * s] = g[97 * s] + x;
    g[100 * s] = g[100 * s] + x;
    g[103 * s] = g[103 * s] + x;
    g[105 * s] = g[105 * s] + x;
    g[108 * s] = g[108 * s] + x;
    g[112 * s] = g[112 * s] + x;
    g[114 * s] = g[114 * s] + x;
    g[116 * s] = g[116 * s] + x;
    g[120 * s] = g[120 * s] + x;
    g[122 * s] = g[122 * s] + x;
    g[124 * s] = g[124 * s] + x;
    g[126 * s] = g[126 * s] + x;
    g[129 * s] = g[129 * s] + x;
    g[131 * s] = g[131 * s] + x;
    g[135 * s] = g[135 * s] + x;
    g[138 * s] = g[138 * s] + x;
    g[142 * s] = g[142 * s] + x;
    g[145 * s] = g[145 * s] + x;
    g[148 * s] = g[148 * s] + x;
    g[152 * s] = g[152 * s] + x;
    g[155 * s] = g[155 * s] + x;
    g[157 * s] = g[157 * s] + x;
    g[160 * s] = g[160 * s] + x;
    g[164 * s] = g[164 * s] + x;
    g[166 * s] = g[166 * s] + x;
    g[168 * s] = g[168 * s] + x;
    g[170 * s] = g[170 * s] + x;
    g[173 * s] = g[173 * s] + x;
    g[175 * s] = g[175 * s] + x;
    g[178 * s] = g[178 * s] + x;
    g[180 * s] = g[180 * s] + x;
    g[182 * s] = g[182 * s] + x;
    g[184 * s] = g[184 * s] + x;
    g[186 * s] = g[186 * s] + x;
    g[188 * s] = g[188 * s] + x;
    g[190 * s] = g[190 * s] + x;
    g[192 * s] = g[192 * s] + x;
    g[194 * s] = g[194 * s] + x;
    g[196 * s] = g[196 * s] + x;
    g[198 * s] = g[198 * s] + x;
    g[200 * s] = g[200 * s] + x;
    g[202 * s] = g[202 * s] + x;
    g[204 * s] = g[204 * s] + x;
    g[206 * s] = g[206 * s] + x;
    g[208 * s] = g[208 * s] + x;
    g[210 * s] = g[210 * s] + x;
    g[212 * s] = g[212 * s] + x;
    g[214 * s] = g[214 * s] + x;
    g[216 * s] = g[216 * s] + x;
    g[218 * s] = g[218 * s] + x;
    g[220 * s] = g[220 * s] + x;
    g[222 * s] = g[222 * s] + x;
    g[224 * s] = g[224 * s] + x;
    g[226 * s] = g[226 * s] + x;
    g[228 * s] = g[228 * s] + x;
    g[231 * s] = g[231 * s] + x;
    g[237 * s] = g[237 * s] + x;
    g[241 * s] = g[241 * s] + x;
    g[244 * s] = g[244 * s] + x;
    g[248 * s] = g[248 * s] + x;
    g[253 * s] = g[253 * s] + x;
    g[255 * s] = g[255 * s] + x;
    g[259 * s] = g[259 * s] + x;
    g[264 * s] = g[264 * s] + x;
    g[267 * s] = g[267 * s] + x;
    g[269 * s] = g[269 * s] + x;
    g[273 * s] = g[273 * s] + x;
    g[279 * s] = g[279 * s] + x;
    g[282 * s] = g[282 * s] + x;
    g[287 * s] = g[287 * s] + x;
    g[296 * s] = g[296 * s] + x;
    g[302 * s] = g[302 * s] + x;
    g[306 * s] = g[306 * s] + x;
    g[310 * s] = g[310 * s] + x;
    g[313 * s] = g[313 * s] + x;
    g[319 * s] = g[319 * s] + x;
    g[326 * s] = g[326 * s] + x;
    g[337 * s] = g[337 * s] + x;
    g[342 * s] = g[342 * s] + x;
    g[345 * s] = g[345 * s] + x;
    g[350 * s] = g[350 * s] + x;
    g[355 * s] = g[355 * s] + x;
    g[360 * s] = g[360 * s] + x;
    g[366 * s] = g[366 * s] + x;
    g[372 * s] = g[372 * s] + x;
    g[378 * s] = g[378 * s] + x;
    g[383 * s] = g[383 * s] + x;
    g[390 * s] = g[390 * s] + x;
    g[396 * s] = g[396 * s] + x;
    g[400 * s] = g[400 * s] + x;
    g[405 * s] = g[405 * s] + x;
    g[410 * s] = g[410 * s] + x;
    g[418 * s] = g[418 * s] + x;
    g[423 * s] = g[423 * s] + x;
    g[431 * s] = g[431 * s] + x;
    g[438 * s] = g[438 * s] + x;
    g[446 * s] = g[446 * s] + x;
    g[452 * s] = g[452 * s] + x;
    g[462 * s] = g[462 * s] + x;
    g[470 * s] = g[470 * s] + x;
    g[480 * s] = g[480 * s] + x;
    g[488 * s] = g[488 * s] + x;
    g[494 * s] = g[494 * s] + x;
    g[505 * s] = g[505 * s] + x;
    g[528 * s] = g[528 * s] + x;
    g[555 * s] = g[555 * s] + x;
    g[584 * s] = g[584 * s] + x;
    g[632 * s] = g[632 * s] + x;
    g[657 * s] = g[657 * s] + x;
    g[669 * s] = g[669 * s] + x;
    g[685 * s] = g[685 * s] + x;
    g[700 * s] = g[700 * s] + x;
    g[737 * s] = g[737 * s] + x;
}

KQ_HD KQ_NOINLINE void kqu_fun_0(const double* v, const double* f, const double* r, double* vdot, long long s)
{
    vdot[0 * s] = 0.0 - (r[32 * s] * v[0 * s]);
    vdot[1 * s] = 0.0 - (r[33 * s] * v[1 * s]);
    vdot[2 * s] = 0.0 - (r[34 * s] * v[2 * s]);
    vdot[3 * s] = 0.0 - (r[35 * s] * v[3 * s]);
    vdot[4 * s] = 0.0 - (r[36 * s] * v[4 * s]);
    vdot[5 * s] = 0.0 - (r[37 * s] * v[5 * s]);
    vdot[6 * s] = 0.0 - (r[38 * s] * v[6 * s]);
    vdot[7 * s] = 0.0 - (r[39 * s] * v[7 * s]);
    vdot[8 * s] = 0.0 + (r[39 * s] * v[7 * s]) - (r[112 * s] * v[8 * s]);
    vdot[9 * s] = 0.0 + (r[37 * s] * v[5 * s]) - (r[113 * s] * v[9 * s]);
    vdot[10 * s] = 0.0 - (r[114 * s] * v[10 * s]);
    vdot[11 * s] = 0.0 + (r[38 * s] * v[6 * s]) - (r[115 * s] * v[11 * s]);
    vdot[12 * s] = 0.0 - (r[120 * s] * v[12 * s]);
    vdot[13 * s] = 0.0 - (r[121 * s] * v[13 * s]);
    vdot[14 * s] = 0.0 - (r[116 * s] * v[14 * s]);
    vdot[15 * s] = 0.0 - (r[117 * s] * v[15 * s]);
    vdot[16 * s] = 0.0 - (r[118 * s] * v[16 * s]);
    vdot[17 * s] = 0.0 + (r[35 * s] * v[3 * s]) - (r[119 * s] * v[17 * s]);
    vdot[18 * s] = 0.0 + (r[95 * s] * v[144 * s]) + (r[124 * s] * v[156 * s]) + (r[125 * s] * v[159 * s]) + (r[262 * s] * v[122 * s]) + (r[263 * s] * v[103 * s]) + (r[264 * s] * v[147 * s]) + (r[265 * s] * v[142 * s]) + (r[266 * s] * v[127 * s]);
    vdot[19 * s] = 0.0 + (r[96 * s] * v[106 * s]);
    vdot[20 * s] = 0.0 + (r[97 * s] * v[124 * s]) + (r[126 * s] * v[114 * s]) + (r[127 * s] * v[113 * s]) + (r[267 * s] * v[21 * s]);
    vdot[21 * s] = 0.0 + (r[201 * s] * v[131 * s] * v[160 * s]) + (r[202 * s] * v[130 * s] * v[160 * s]) - (r[267 * s] * v[21 * s]);
    vdot[22 * s] = 0.0 + (r[98 * s] * v[107 * s]);
    vdot[23 * s] = 0.0 + (r[99 * s] * v[145 * s]);
    vdot[24 * s] = 0.0 + (r[100 * s] * v[157 * s]);
    vdot[25 * s] = 0.0 + (r[101 * s] * v[141 * s]) + (r[128 * s] * v[137 * s]);
    vdot[26 * s] = 0.0 + (r[102 * s] * v[120 * s]);
    vdot[27 * s] = 0.0 + (r[103 * s] * v[121 * s]);
    vdot[28 * s] = 0.0 + (r[104 * s] * v[109 * s]) + (r[108 * s] * v[153 * s]) + (r[129 * s] * v[123 * s]);
    vdot[29 * s] = 0.0 + (r[105 * s] * v[110 * s]);
    vdot[30 * s] = 0.0 + (r[106 * s] * v[105 * s]);
    vdot[31 * s] = 0.0 + (r[107 * s] * v[112 * s]);
    vdot[32 * s] = 0.0 + (r[139 * s] * v[160 * s]);
    vdot[33 * s] = 0.0 + (r[109 * s] * v[146 * s]);
    vdot[34 * s] = 0.0 + (r[110 * s] * v[108 * s]);
    vdot[35 * s] = 0.0 + (r[111 * s] * v[111 * s]);
    vdot[36 * s] = 0.0 + (r[112 * s] * v[8 * s]);
    vdot[37 * s] = 0.0 + (r[120 * s] * v[12 * s]);
    vdot[38 * s] = 0.0 + (r[121 * s] * v[13 * s]);
    vdot[39 * s] = 0.0 + (r[113 * s] * v[9 * s]);
    vdot[40 * s] = 0.0 + (r[114 * s] * v[10 * s]);
    vdot[41 * s] = 0.0 + (r[115 * s] * v[11 * s]);
    vdot[42 * s] = 0.0 + (r[122 * s] * v[155 * s]);
    vdot[43 * s] = 0.0 + (r[116 * s] * v[14 * s]);
    vdot[44 * s] = 0.0 + (r[117 * s] * v[15 * s]);
    vdot[45 * s] = 0.0 + (r[118 * s] * v[16 * s]);
    vdot[46 * s] = 0.0 + (r[119 * s] * v[17 * s]);
    vdot[47 * s] = 0.0 + (r[132 * s] * v[158 * s]);
    vdot[48 * s] = 0.0 + (r[133 * s] * v[125 * s]) + (r[134 * s] * v[151 * s]);
    vdot[49 * s] = 0.0 + (r[135 * s] * v[129 * s]) + (r[136 * s] * v[149 * s]);
    vdot[50 * s] = 0.0 + (r[157 * s] * v[115 * s]);
    vdot[51 * s] = 0.0 + (r[158 * s] * v[101 * s]) + (r[165 * s] * v[52 * s]);
    vdot[52 * s] = 0.0 + (r[150 * s] * v[115 * s] * f[0 * s]) + (r[151 * s] * v[115 * s] * v[153 * s]) + (r[152 * s] * v[115 * s] * v[146 * s]) - (r[165 * s] * v[52 * s]);
    vdot[53 * s] = 0.0 + (r[159 * s] * v[102 * s]);
    vdot[54 * s] = 0.0 + (r[160 * s] * v[55 * s]);
    vdot[55 * s] = 0.0 + (r[148 * s] * v[101 * s] * v[115 * s]) + (r[149 * s] * v[102 * s] * v[115 * s]) - (r[160 * s] * v[55 * s]);
    vdot[56 * s] = 0.0 + (r[161 * s] * v[75 * s]);
    vdot[57 * s] = 0.0 + (r[162 * s] * v[77 * s]);
    vdot[58 * s] = 0.0 + (r[163 * s] * v[59 * s]);
    vdot[59 * s] = 0.0 + (r[153 * s] * v[75 * s] * f[0 * s]) + (r[155 * s] * v[77 * s] * f[0 * s]) - (r[163 * s] * v[59 * s]);
    vdot[60 * s] = 0.0 + (r[164 * s] * v[61 * s]);
    vdot[61 * s] = 0.0 + (r[154 * s] * v[75 * s] * v[153 * s]) + (r[156 * s] * v[77 * s] * v[153 * s]) - (r[164 * s] * v[61 * s]);
}

KQ_HD KQ_NOINLINE void kqu_fun_1(const double* v, const double* f, const double* r, double* vdot, long long s)
{
    vdot[62 * s] = 0.0 + (r[211 * s] * v[136 * s]) + (r[212 * s] * v[140 * s]);
    vdot[63 * s] = 0.0 + (r[213 * s] * v[128 * s]) + (r[214 * s] * v[131 * s]) + (r[215 * s] * v[130 * s]);
    vdot[64 * s] = 0.0 + (r[216 * s] * v[133 * s]) + (r[217 * s] * v[132 * s]);
    vdot[65 * s] = 0.0 + (r[218 * s] * v[134 * s]) + (r[219 * s] * v[135 * s]);
    vdot[66 * s] = 0.0 + (r[220 * s] * v[148 * s]) + (r[224 * s] * v[143 * s]) + (r[264 * s] * v[147 * s]);
    vdot[67 * s] = 0.0 + (r[130 * s] * v[150 * s]) + (r[131 * s] * v[154 * s]);
    vdot[68 * s] = 0.0 + (r[221 * s] * v[104 * s]);
    vdot[69 * s] = 0.0 + (r[222 * s] * v[138 * s]) + (r[223 * s] * v[139 * s]);
    vdot[70 * s] = 0.0 + (r[225 * s] * v[118 * s]) + (r[226 * s] * v[116 * s]) + (r[268 * s] * v[117 * s]);
    vdot[71 * s] = 0.0 + (r[260 * s] * v[126 * s]);
    vdot[72 * s] = 0.0 + (r[261 * s] * v[119 * s]);
    vdot[73 * s] = 0.0 - (r[14 * s] * v[73 * s]) + (r[30 * s] * v[125 * s]);
    vdot[74 * s] = 0.0 - (r[141 * s] * v[74 * s]) + (r[144 * s] * v[75 * s]);
    vdot[75 * s] = 0.0 + (r[141 * s] * v[74 * s]) - (r[144 * s] * v[75 * s]) - (r[153 * s] * v[75 * s] * f[0 * s]) - (r[154 * s] * v[75 * s] * v[153 * s]) - (r[161 * s] * v[75 * s]);
    vdot[76 * s] = 0.0 - (r[142 * s] * v[76 * s]) + (r[145 * s] * v[77 * s]);
    vdot[77 * s] = 0.0 + (r[142 * s] * v[76 * s]) - (r[145 * s] * v[77 * s]) - (r[155 * s] * v[77 * s] * f[0 * s]) - (r[156 * s] * v[77 * s] * v[153 * s]) - (r[162 * s] * v[77 * s]);
    vdot[78 * s] = 0.0 - (r[166 * s] * v[78 * s]) + (r[171 * s] * v[104 * s]);
    vdot[79 * s] = 0.0 - (r[167 * s] * v[79 * s]) + (r[172 * s] * v[134 * s]);
    vdot[80 * s] = 0.0 - (r[168 * s] * v[80 * s]) + (r[173 * s] * v[143 * s]);
    vdot[81 * s] = 0.0 - (r[12 * s] * v[81 * s]) + (r[28 * s] * v[154 * s]);
    vdot[82 * s] = 0.0 - (r[170 * s] * v[82 * s]) + (r[175 * s] * v[133 * s]);
    vdot[83 * s] = 0.0 - (r[169 * s] * v[83 * s]) + (r[174 * s] * v[118 * s]);
    vdot[84 * s] = 0.0 - (r[4 * s] * v[84 * s]) + (r[20 * s] * v[145 * s]);
    vdot[85 * s] = 0.0 - (r[1 * s] * v[85 * s]) + (r[17 * s] * v[106 * s]);
    vdot[86 * s] = 0.0 - (r[2 * s] * v[86 * s]) + (r[18 * s] * v[124 * s]);
    vdot[87 * s] = 0.0 - (r[3 * s] * v[87 * s]) + (r[19 * s] * v[107 * s]);
    vdot[88 * s] = 0.0 - (r[5 * s] * v[88 * s]) + (r[21 * s] * v[157 * s]);
    vdot[89 * s] = 0.0 - (r[6 * s] * v[89 * s]) + (r[22 * s] * v[141 * s]);
    vdot[90 * s] = 0.0 - (r[7 * s] * v[90 * s]) + (r[23 * s] * v[120 * s]);
    vdot[91 * s] = 0.0 - (r[8 * s] * v[91 * s]) + (r[24 * s] * v[121 * s]);
    vdot[92 * s] = 0.0 - (r[9 * s] * v[92 * s]) + (r[25 * s] * v[110 * s]);
    vdot[93 * s] = 0.0 - (r[10 * s] * v[93 * s]) + (r[26 * s] * v[105 * s]);
    vdot[94 * s] = 0.0 - (r[11 * s] * v[94 * s]) + (r[27 * s] * v[112 * s]);
    vdot[95 * s] = 0.0 - (r[13 * s] * v[95 * s]) + (r[29 * s] * v[158 * s]);
    vdot[96 * s] = 0.0 - (r[15 * s] * v[96 * s]) + (r[31 * s] * v[149 * s]);
    vdot[97 * s] = 0.0 - (r[227 * s] * v[97 * s]) + (r[229 * s] * v[126 * s]);
    vdot[98 * s] = 0.0 - (r[228 * s] * v[98 * s]) + (r[230 * s] * v[119 * s]);
    vdot[99 * s] = 0.0 - (r[0 * s] * v[99 * s]) + (r[16 * s] * v[144 * s]);
    vdot[100 * s] = 0.0 - (r[140 * s] * v[100 * s]) + (r[143 * s] * v[115 * s]);
    vdot[101 * s] = 0.0 + (r[146 * s] * v[115 * s] * f[0 * s]) - (r[148 * s] * v[101 * s] * v[115 * s]) - (r[158 * s] * v[101 * s]);
    vdot[102 * s] = 0.0 + (r[147 * s] * v[115 * s] * v[153 * s]) - (r[149 * s] * v[102 * s] * v[115 * s]) - (r[159 * s] * v[102 * s]);
}

KQ_HD KQ_NOINLINE void kqu_fun_2(const double* v, const double* f, const double* r, double* vdot, long long s)
{
    vdot[103 * s] = 0.0 + (r[236 * s] * v[156 * s] * v[160 * s]) + (r[241 * s] * v[126 * s] * v[156 * s]) - (r[242 * s] * v[103 * s] * f[2 * s]) + (r[248 * s] * v[119 * s] * v[156 * s]) - (r[263 * s] * v[103 * s]);
    vdot[104 * s] = 0.0 + (r[166 * s] * v[78 * s]) - (r[171 * s] * v[104 * s]) - (r[193 * s] * v[104 * s] * v[160 * s]) - (r[194 * s] * v[104 * s] * v[160 * s]) - (r[221 * s] * v[104 * s]);
    vdot[105 * s] = 0.0 + (r[10 * s] * v[93 * s]) - (r[26 * s] * v[105 * s]) - (r[106 * s] * v[105 * s]) + (r[194 * s] * v[104 * s] * v[160 * s]) - (r[197 * s] * v[105 * s] * v[160 * s]);
    vdot[106 * s] = 0.0 + (r[1 * s] * v[85 * s]) - (r[17 * s] * v[106 * s]) - (r[42 * s] * v[106 * s]) + (r[56 * s] * v[146 * s] * v[155 * s]) - (r[96 * s] * v[106 * s]);
    vdot[107 * s] = 0.0 + (r[3 * s] * v[87 * s]) - (r[19 * s] * v[107 * s]) - (r[45 * s] * v[107 * s]) + (r[59 * s] * v[108 * s] * v[152 * s]) - (r[98 * s] * v[107 * s]);
    vdot[108 * s] = 0.0 + (r[33 * s] * v[1 * s]) + (r[45 * s] * v[107 * s]) - (r[59 * s] * v[108 * s] * v[152 * s]) - (r[110 * s] * v[108 * s]);
    vdot[109 * s] = 0.0 - (r[49 * s] * v[109 * s]) + (r[63 * s] * v[123 * s] * v[155 * s]) - (r[104 * s] * v[109 * s]);
    vdot[110 * s] = 0.0 + (r[9 * s] * v[92 * s]) - (r[25 * s] * v[110 * s]) - (r[47 * s] * v[110 * s]) + (r[61 * s] * v[111 * s] * v[155 * s]) - (r[105 * s] * v[110 * s]);
    vdot[111 * s] = 0.0 + (r[34 * s] * v[2 * s]) + (r[47 * s] * v[110 * s]) - (r[61 * s] * v[111 * s] * v[155 * s]) - (r[111 * s] * v[111 * s]);
    vdot[112 * s] = 0.0 + (r[11 * s] * v[94 * s]) - (r[27 * s] * v[112 * s]) - (r[107 * s] * v[112 * s]) - (r[203 * s] * v[112 * s] * v[160 * s]);
    vdot[113 * s] = 0.0 + (r[44 * s] * v[114 * s]) - (r[58 * s] * v[113 * s] * v[155 * s]) - (r[127 * s] * v[113 * s]);
    vdot[114 * s] = 0.0 + (r[43 * s] * v[124 * s]) - (r[44 * s] * v[114 * s]) - (r[57 * s] * v[114 * s] * v[155 * s]) + (r[58 * s] * v[113 * s] * v[155 * s]) - (r[126 * s] * v[114 * s]);
    vdot[115 * s] = 0.0 + (r[140 * s] * v[100 * s]) - (r[143 * s] * v[115 * s]) - (r[146 * s] * v[115 * s] * f[0 * s]) - (r[147 * s] * v[115 * s] * v[153 * s]) - (r[148 * s] * v[101 * s] * v[115 * s]) - (r[149 * s] * v[102 * s] * v[115 * s]) - (r[150 * s] * v[115 * s] * f[0 * s]) - (r[151 * s] * v[115 * s] * v[153 * s]) - (r[152 * s] * v[115 * s] * v[146 * s]) - (r[157 * s] * v[115 * s]);
    vdot[116 * s] = 0.0 + (r[190 * s] * v[118 * s] * f[0 * s]) - (r[191 * s] * v[116 * s]) - (r[210 * s] * v[116 * s] * v[160 * s]) - (r[226 * s] * v[116 * s]) + (r[258 * s] * v[117 * s] * v[152 * s]);
    vdot[117 * s] = 0.0 + (r[255 * s] * v[118 * s] * v[156 * s]) + (r[256 * s] * v[118 * s] * v[159 * s]) - (r[257 * s] * v[117 * s]) - (r[258 * s] * v[117 * s] * v[152 * s]) - (r[259 * s] * v[117 * s] * v[160 * s]) - (r[268 * s] * v[117 * s]);
    vdot[118 * s] = 0.0 + (r[169 * s] * v[83 * s]) - (r[174 * s] * v[118 * s]) - (r[190 * s] * v[118 * s] * f[0 * s]) + (r[191 * s] * v[116 * s]) - (r[225 * s] * v[118 * s]) - (r[255 * s] * v[118 * s] * v[156 * s]) - (r[256 * s] * v[118 * s] * v[159 * s]) + (r[257 * s] * v[117 * s]);
}

KQ_HD KQ_NOINLINE void kqu_fun_3(const double* v, const double* f, const double* r, double* vdot, long long s)
{
    vdot[119 * s] = 0.0 + (r[228 * s] * v[98 * s]) - (r[230 * s] * v[119 * s]) + -0x1.0000000000000p+1 * (r[247 * s] * v[119 * s] * v[119 * s]) - (r[248 * s] * v[119 * s] * v[156 * s]) - (r[261 * s] * v[119 * s]);
    vdot[120 * s] = 0.0 + (r[7 * s] * v[90 * s]) - (r[23 * s] * v[120 * s]) - (r[81 * s] * v[120 * s] * v[155 * s] * v[156 * s]) - (r[102 * s] * v[120 * s]) + (r[248 * s] * v[119 * s] * v[156 * s]);
    vdot[121 * s] = 0.0 + (r[8 * s] * v[91 * s]) - (r[24 * s] * v[121 * s]) - (r[82 * s] * v[121 * s] * v[155 * s] * v[156 * s]) - (r[83 * s] * v[121 * s] * v[156 * s]) - (r[103 * s] * v[121 * s]);
    vdot[122 * s] = 0.0 + (r[240 * s] * v[126 * s] * v[153 * s]) + 0x1.0000000000000p+1 * (r[244 * s] * v[142 * s] * v[142 * s]) - (r[246 * s] * v[122 * s] * f[0 * s]) - (r[262 * s] * v[122 * s]);
    vdot[123 * s] = 0.0 + (r[49 * s] * v[109 * s]) - (r[50 * s] * v[123 * s]) - (r[63 * s] * v[123 * s] * v[155 * s]) + (r[64 * s] * v[153 * s] * v[155 * s]) - (r[129 * s] * v[123 * s]) + (r[246 * s] * v[122 * s] * f[0 * s]);
    vdot[124 * s] = 0.0 + (r[2 * s] * v[86 * s]) - (r[18 * s] * v[124 * s]) - (r[43 * s] * v[124 * s]) + (r[57 * s] * v[114 * s] * v[155 * s]) - (r[97 * s] * v[124 * s]) + 0x1.0000000000000p+1 * (r[200 * s] * v[128 * s] * v[160 * s]) + (r[201 * s] * v[131 * s] * v[160 * s]) + (r[202 * s] * v[130 * s] * v[160 * s]) + (r[204 * s] * v[133 * s] * v[160 * s]) + (r[205 * s] * v[132 * s] * v[160 * s]) + (r[209 * s] * v[141 * s] * v[160 * s]) + (r[249 * s] * v[137 * s] * v[160 * s]);
    vdot[125 * s] = 0.0 + (r[14 * s] * v[73 * s]) - (r[30 * s] * v[125 * s]) - (r[52 * s] * v[125 * s]) + (r[66 * s] * v[151 * s] * v[155 * s]) - (r[94 * s] * v[125 * s] * v[160 * s]) - (r[133 * s] * v[125 * s]);
    vdot[126 * s] = 0.0 + (r[227 * s] * v[97 * s]) - (r[229 * s] * v[126 * s]) - (r[240 * s] * v[126 * s] * v[153 * s]) - (r[241 * s] * v[126 * s] * v[156 * s]) - (r[260 * s] * v[126 * s]);
    vdot[127 * s] = 0.0 + (r[243 * s] * v[142 * s] * v[154 * s]) - (r[245 * s] * v[127 * s] * v[155 * s] * v[156 * s]) - (r[266 * s] * v[127 * s]);
    vdot[128 * s] = 0.0 - (r[177 * s] * v[128 * s]) + (r[183 * s] * v[131 * s] * v[155 * s]) + (r[198 * s] * v[136 * s] * v[160 * s]) - (r[200 * s] * v[128 * s] * v[160 * s]) - (r[213 * s] * v[128 * s]);
    vdot[129 * s] = 0.0 + (r[53 * s] * v[149 * s]) - (r[67 * s] * v[129 * s] * v[155 * s]) - (r[91 * s] * v[129 * s]) - (r[135 * s] * v[129 * s]) + (r[238 * s] * v[150 * s] * v[158 * s]);
    vdot[130 * s] = 0.0 + (r[178 * s] * v[131 * s]) - (r[184 * s] * v[130 * s] * v[155 * s]) - (r[202 * s] * v[130 * s] * v[160 * s]) - (r[215 * s] * v[130 * s]);
    vdot[131 * s] = 0.0 + (r[177 * s] * v[128 * s]) - (r[178 * s] * v[131 * s]) - (r[183 * s] * v[131 * s] * v[155 * s]) + (r[184 * s] * v[130 * s] * v[155 * s]) + (r[199 * s] * v[140 * s] * v[160 * s]) - (r[201 * s] * v[131 * s] * v[160 * s]) - (r[214 * s] * v[131 * s]);
    vdot[132 * s] = 0.0 + (r[179 * s] * v[133 * s]) - (r[185 * s] * v[132 * s] * v[155 * s]) + 0x1.d70a3e0000000p-1 * (r[203 * s] * v[112 * s] * v[160 * s]) - (r[205 * s] * v[132 * s] * v[160 * s]) - (r[217 * s] * v[132 * s]);
}

KQ_HD KQ_NOINLINE void kqu_fun_4(const double* v, const double* f, const double* r, double* vdot, long long s)
{
    vdot[133 * s] = 0.0 + (r[170 * s] * v[82 * s]) - (r[175 * s] * v[133 * s]) - (r[179 * s] * v[133 * s]) + (r[185 * s] * v[132 * s] * v[155 * s]) - (r[204 * s] * v[133 * s] * v[160 * s]) - (r[216 * s] * v[133 * s]);
    vdot[134 * s] = 0.0 + (r[167 * s] * v[79 * s]) - (r[172 * s] * v[134 * s]) - (r[181 * s] * v[134 * s]) + (r[187 * s] * v[135 * s] * v[155 * s]) + (r[204 * s] * v[133 * s] * v[160 * s]) - (r[206 * s] * v[134 * s] * v[160 * s]) - (r[218 * s] * v[134 * s]);
    vdot[135 * s] = 0.0 + (r[181 * s] * v[134 * s]) - (r[187 * s] * v[135 * s] * v[155 * s]) + (r[205 * s] * v[132 * s] * v[160 * s]) - (r[207 * s] * v[135 * s] * v[160 * s]) - (r[219 * s] * v[135 * s]);
    vdot[136 * s] = 0.0 - (r[176 * s] * v[136 * s]) + (r[182 * s] * v[140 * s] * v[155 * s]) + (r[197 * s] * v[105 * s] * v[160 * s]) - (r[198 * s] * v[136 * s] * v[160 * s]) + 0x1.b333340000000p-1 * (r[206 * s] * v[134 * s] * v[160 * s]) - (r[211 * s] * v[136 * s]);
    vdot[137 * s] = 0.0 + (r[46 * s] * v[141 * s]) - (r[60 * s] * v[137 * s] * v[155 * s]) - (r[128 * s] * v[137 * s]) - (r[249 * s] * v[137 * s] * v[160 * s]);
    vdot[138 * s] = 0.0 - (r[180 * s] * v[138 * s]) + (r[186 * s] * v[139 * s] * v[155 * s]) + (r[193 * s] * v[104 * s] * v[160 * s]) - (r[195 * s] * v[138 * s] * v[160 * s]) - (r[222 * s] * v[138 * s]);
    vdot[139 * s] = 0.0 + (r[180 * s] * v[138 * s]) - (r[186 * s] * v[139 * s] * v[155 * s]) - (r[196 * s] * v[139 * s] * v[160 * s]) - (r[223 * s] * v[139 * s]);
    vdot[140 * s] = 0.0 + (r[176 * s] * v[136 * s]) - (r[182 * s] * v[140 * s] * v[155 * s]) + (r[195 * s] * v[138 * s] * v[160 * s]) + (r[196 * s] * v[139 * s] * v[160 * s]) - (r[199 * s] * v[140 * s] * v[160 * s]) + 0x1.47ae140000000p-4 * (r[203 * s] * v[112 * s] * v[160 * s]) + 0x1.b333340000000p-1 * (r[207 * s] * v[135 * s] * v[160 * s]) - (r[212 * s] * v[140 * s]);
    vdot[141 * s] = 0.0 + (r[6 * s] * v[89 * s]) - (r[22 * s] * v[141 * s]) - (r[46 * s] * v[141 * s]) + (r[60 * s] * v[137 * s] * v[155 * s]) - (r[101 * s] * v[141 * s]) + (r[208 * s] * v[148 * s] * v[160 * s]) - (r[209 * s] * v[141 * s] * v[160 * s]) + (r[254 * s] * v[147 * s] * v[160 * s]);
    vdot[142 * s] = 0.0 + (r[242 * s] * v[103 * s] * f[2 * s]) - (r[243 * s] * v[142 * s] * v[154 * s]) + -0x1.0000000000000p+1 * (r[244 * s] * v[142 * s] * v[142 * s]) - (r[265 * s] * v[142 * s]);
    vdot[143 * s] = 0.0 + (r[168 * s] * v[80 * s]) - (r[173 * s] * v[143 * s]) - (r[188 * s] * v[143 * s] * f[0 * s]) + (r[189 * s] * v[148 * s]) - (r[224 * s] * v[143 * s]) + 0x1.0000000000000p+1 * (r[247 * s] * v[119 * s] * v[119 * s]) - (r[250 * s] * v[143 * s] * v[156 * s]) - (r[251 * s] * v[143 * s] * v[159 * s]) + (r[252 * s] * v[147 * s]);
    vdot[144 * s] = 0.0 + (r[0 * s] * v[99 * s]) - (r[16 * s] * v[144 * s]) - (r[40 * s] * v[144 * s]) + (r[54 * s] * v[155 * s] * v[156 * s]) - (r[69 * s] * v[144 * s] * v[157 * s]) - (r[72 * s] * v[13 * s] * v[144 * s]) - (r[75 * s] * v[12 * s] * v[144 * s]) - (r[78 * s] * v[12 * s] * v[13 * s] * v[144 * s]) - (r[87 * s] * v[144 * s] * v[158 * s]) - (r[95 * s] * v[144 * s]);
}

KQ_HD KQ_NOINLINE void kqu_fun_5(const double* v, const double* f, const double* r, double* vdot, long long s)
{
    vdot[145 * s] = 0.0 + (r[4 * s] * v[84 * s]) - (r[20 * s] * v[145 * s]) - (r[68 * s] * v[145 * s] * v[155 * s] * v[156 * s]) + (r[84 * s] * v[154 * s] * v[154 * s]) + (r[85 * s] * v[150 * s] * v[154 * s]) - (r[99 * s] * v[145 * s]) - (r[192 * s] * v[145 * s]) + (r[232 * s] * v[160 * s] * v[160 * s]) - (r[235 * s] * v[145 * s] * v[160 * s]);
    vdot[146 * s] = 0.0 + (r[32 * s] * v[0 * s]) + (r[42 * s] * v[106 * s]) - (r[56 * s] * v[146 * s] * v[155 * s]) + (r[90 * s] * v[149 * s] * v[156 * s]) + (r[92 * s] * v[151 * s] * v[157 * s]) - (r[109 * s] * v[146 * s]) - (r[152 * s] * v[115 * s] * v[146 * s]) - (r[231 * s] * v[146 * s]) + (r[240 * s] * v[126 * s] * v[153 * s]) + (r[241 * s] * v[126 * s] * v[156 * s]);
    vdot[147 * s] = 0.0 + (r[250 * s] * v[143 * s] * v[156 * s]) + (r[251 * s] * v[143 * s] * v[159 * s]) - (r[252 * s] * v[147 * s]) - (r[253 * s] * v[147 * s] * v[152 * s]) - (r[254 * s] * v[147 * s] * v[160 * s]) - (r[264 * s] * v[147 * s]);
    vdot[148 * s] = 0.0 + (r[188 * s] * v[143 * s] * f[0 * s]) - (r[189 * s] * v[148 * s]) + 0x1.3333340000000p-3 * (r[206 * s] * v[134 * s] * v[160 * s]) + 0x1.3333340000000p-3 * (r[207 * s] * v[135 * s] * v[160 * s]) - (r[208 * s] * v[148 * s] * v[160 * s]) - (r[220 * s] * v[148 * s]) + (r[253 * s] * v[147 * s] * v[152 * s]);
    vdot[149 * s] = 0.0 + (r[15 * s] * v[96 * s]) - (r[31 * s] * v[149 * s]) - (r[53 * s] * v[149 * s]) + (r[67 * s] * v[129 * s] * v[155 * s]) - (r[90 * s] * v[149 * s] * v[156 * s]) - (r[136 * s] * v[149 * s]) + (r[237 * s] * v[154 * s] * v[158 * s]) - (r[239 * s] * v[149 * s]);
    vdot[150 * s] = 0.0 + (r[51 * s] * v[154 * s]) - (r[65 * s] * v[150 * s] * v[155 * s]) - (r[85 * s] * v[150 * s] * v[154 * s]) - (r[86 * s] * v[150 * s] * v[157 * s]) - (r[130 * s] * v[150 * s]) - (r[234 * s] * v[150 * s] * v[160 * s]) - (r[238 * s] * v[150 * s] * v[158 * s]);
    vdot[151 * s] = 0.0 + (r[52 * s] * v[125 * s]) - (r[66 * s] * v[151 * s] * v[155 * s]) + 0x1.0000000000000p+1 * (r[87 * s] * v[144 * s] * v[158 * s]) + 0x1.0000000000000p+1 * (r[88 * s] * v[156 * s] * v[158 * s]) + 0x1.0000000000000p+1 * (r[89 * s] * v[158 * s] * v[159 * s]) + (r[91 * s] * v[129 * s]) - (r[92 * s] * v[151 * s] * v[157 * s]) - (r[93 * s] * v[151 * s] * v[160 * s]) - (r[134 * s] * v[151 * s]);
    vdot[152 * s] = 0.0 + (r[45 * s] * v[107 * s]) + (r[48 * s] * f[0 * s]) - (r[59 * s] * v[108 * s] * v[152 * s]) - (r[62 * s] * v[152 * s] * v[155 * s]) + (r[85 * s] * v[150 * s] * v[154 * s]) + (r[86 * s] * v[150 * s] * v[157 * s]) + (r[93 * s] * v[151 * s] * v[160 * s]) - (r[123 * s] * v[152 * s]) + (r[202 * s] * v[130 * s] * v[160 * s]) + (r[231 * s] * v[146 * s]) + (r[234 * s] * v[150 * s] * v[160 * s]) + (r[249 * s] * v[137 * s] * v[160 * s]) + (r[251 * s] * v[143 * s] * v[159 * s]) - (r[253 * s] * v[147 * s] * v[152 * s]);
}

KQ_HD KQ_NOINLINE void kqu_fun_6(const double* v, const double* f, const double* r, double* vdot, long long s)
{
    vdot[153 * s] = 0.0 + (r[36 * s] * v[4 * s]) + (r[50 * s] * v[123 * s]) - (r[64 * s] * v[153 * s] * v[155 * s]) + (r[68 * s] * v[145 * s] * v[155 * s] * v[156 * s]) + (r[69 * s] * v[144 * s] * v[157 * s]) + (r[70 * s] * v[156 * s] * v[157 * s]) + (r[71 * s] * v[157 * s] * v[159 * s]) + (r[72 * s] * v[13 * s] * v[144 * s]) + (r[73 * s] * v[13 * s] * v[156 * s]) + (r[74 * s] * v[13 * s] * v[159 * s]) + (r[75 * s] * v[12 * s] * v[144 * s]) + (r[76 * s] * v[12 * s] * v[156 * s]) + (r[77 * s] * v[12 * s] * v[159 * s]) + (r[78 * s] * v[12 * s] * v[13 * s] * v[144 * s]) + (r[79 * s] * v[12 * s] * v[13 * s] * v[156 * s]) + (r[80 * s] * v[12 * s] * v[13 * s] * v[159 * s]) + (r[81 * s] * v[120 * s] * v[155 * s] * v[156 * s]) + (r[82 * s] * v[121 * s] * v[155 * s] * v[156 * s]) + (r[83 * s] * v[121 * s] * v[156 * s]) + (r[87 * s] * v[144 * s] * v[158 * s]) + (r[88 * s] * v[156 * s] * v[158 * s]) + (r[89 * s] * v[158 * s] * v[159 * s]) + (r[90 * s] * v[149 * s] * v[156 * s]) - (r[108 * s] * v[153 * s]) - (r[147 * s] * v[115 * s] * v[153 * s]) - (r[151 * s] * v[115 * s] * v[153 * s]) - (r[154 * s] * v[75 * s] * v[153 * s]) - (r[156 * s] * v[77 * s] * v[153 * s]) - (r[240 * s] * v[126 * s] * v[153 * s]) + 0x1.0000000000000p+1 * (r[245 * s] * v[127 * s] * v[155 * s] * v[156 * s]);
    vdot[154 * s] = 0.0 + (r[12 * s] * v[81 * s]) - (r[28 * s] * v[154 * s]) - (r[51 * s] * v[154 * s]) + (r[65 * s] * v[150 * s] * v[155 * s]) + -0x1.0000000000000p+1 * (r[84 * s] * v[154 * s] * v[154 * s]) - (r[85 * s] * v[150 * s] * v[154 * s]) - (r[131 * s] * v[154 * s]) + (r[193 * s] * v[104 * s] * v[160 * s]) + (r[194 * s] * v[104 * s] * v[160 * s]) + (r[195 * s] * v[138 * s] * v[160 * s]) + (r[196 * s] * v[139 * s] * v[160 * s]) + (r[197 * s] * v[105 * s] * v[160 * s]) + (r[198 * s] * v[136 * s] * v[160 * s]) + (r[199 * s] * v[140 * s] * v[160 * s]) + (r[203 * s] * v[112 * s] * v[160 * s]) + (r[204 * s] * v[133 * s] * v[160 * s]) + (r[205 * s] * v[132 * s] * v[160 * s]) + (r[208 * s] * v[148 * s] * v[160 * s]) + (r[209 * s] * v[141 * s] * v[160 * s]) - (r[233 * s] * v[154 * s] * v[160 * s]) + (r[235 * s] * v[145 * s] * v[160 * s]) - (r[237 * s] * v[154 * s] * v[158 * s]) + (r[239 * s] * v[149 * s]) - (r[243 * s] * v[142 * s] * v[154 * s]) + 0x1.0000000000000p+1 * (r[247 * s] * v[119 * s] * v[119 * s]) + (r[249 * s] * v[137 * s] * v[160 * s]) + (r[254 * s] * v[147 * s] * v[160 * s]);
}

KQ_HD KQ_NOINLINE void kqu_fun_7(const double* v, const double* f, const double* r, double* vdot, long long s)
{
    vdot[155 * s] = 0.0 + (r[40 * s] * v[144 * s]) + (r[41 * s] * v[156 * s]) + (r[42 * s] * v[106 * s]) + (r[43 * s] * v[124 * s]) + (r[44 * s] * v[114 * s]) + (r[46 * s] * v[141 * s]) + (r[47 * s] * v[110 * s]) + (r[48 * s] * f[0 * s]) + (r[49 * s] * v[109 * s]) + (r[50 * s] * v[123 * s]) + (r[51 * s] * v[154 * s]) + (r[52 * s] * v[125 * s]) + (r[53 * s] * v[149 * s]) - (r[54 * s] * v[155 * s] * v[156 * s]) - (r[55 * s] * v[155 * s] * v[159 * s]) - (r[56 * s] * v[146 * s] * v[155 * s]) - (r[57 * s] * v[114 * s] * v[155 * s]) - (r[58 * s] * v[113 * s] * v[155 * s]) - (r[60 * s] * v[137 * s] * v[155 * s]) - (r[61 * s] * v[111 * s] * v[155 * s]) - (r[62 * s] * v[152 * s] * v[155 * s]) - (r[63 * s] * v[123 * s] * v[155 * s]) - (r[64 * s] * v[153 * s] * v[155 * s]) - (r[65 * s] * v[150 * s] * v[155 * s]) - (r[66 * s] * v[151 * s] * v[155 * s]) - (r[67 * s] * v[129 * s] * v[155 * s]) + (r[68 * s] * v[145 * s] * v[155 * s] * v[156 * s]) + 0x1.0000000000000p+1 * (r[69 * s] * v[144 * s] * v[157 * s]) + (r[70 * s] * v[156 * s] * v[157 * s]) + 0x1.0000000000000p+1 * (r[72 * s] * v[13 * s] * v[144 * s]) + (r[73 * s] * v[13 * s] * v[156 * s]) + 0x1.0000000000000p+1 * (r[75 * s] * v[12 * s] * v[144 * s]) + (r[76 * s] * v[12 * s] * v[156 * s]) + 0x1.0000000000000p+1 * (r[78 * s] * v[12 * s] * v[13 * s] * v[144 * s]) + (r[79 * s] * v[12 * s] * v[13 * s] * v[156 * s]) + (r[81 * s] * v[120 * s] * v[155 * s] * v[156 * s]) + (r[82 * s] * v[121 * s] * v[155 * s] * v[156 * s]) + (r[83 * s] * v[121 * s] * v[156 * s]) + 0x1.0000000000000p+2 * (r[87 * s] * v[144 * s] * v[158 * s]) + 0x1.8000000000000p+1 * (r[88 * s] * v[156 * s] * v[158 * s]) + 0x1.0000000000000p+1 * (r[89 * s] * v[158 * s] * v[159 * s]) + 0x1.0000000000000p+1 * (r[90 * s] * v[149 * s] * v[156 * s]) - (r[122 * s] * v[155 * s]) + (r[176 * s] * v[136 * s]) + (r[177 * s] * v[128 * s]) + (r[178 * s] * v[131 * s]) + (r[179 * s] * v[133 * s]) + (r[180 * s] * v[138 * s]) + (r[181 * s] * v[134 * s]) - (r[182 * s] * v[140 * s] * v[155 * s]) - (r[183 * s] * v[131 * s] * v[155 * s]) - (r[184 * s] * v[130 * s] * v[155 * s]) - (r[185 * s] * v[132 * s] * v[155 * s]) - (r[186 * s] * v[139 * s] * v[155 * s]) - (r[187 * s] * v[135 * s] * v[155 * s]) + (r[195 * s] * v[138 * s] * v[160 * s]) + (r[241 * s] * v[126 * s] * v[156 * s]) + 0x1.0000000000000p+1 * (r[245 * s] * v[127 * s] * v[155 * s] * v[156 * s]);
}

KQ_HD KQ_NOINLINE void kqu_fun_8(const double* v, const double* f, const double* r, double* vdot, long long s)
{
    vdot[156 * s] = 0.0 + (r[40 * s] * v[144 * s]) - (r[41 * s] * v[156 * s]) - (r[54 * s] * v[155 * s] * v[156 * s]) + (r[55 * s] * v[155 * s] * v[159 * s]) - (r[68 * s] * v[145 * s] * v[155 * s] * v[156 * s]) - (r[70 * s] * v[156 * s] * v[157 * s]) - (r[73 * s] * v[13 * s] * v[156 * s]) - (r[76 * s] * v[12 * s] * v[156 * s]) - (r[79 * s] * v[12 * s] * v[13 * s] * v[156 * s]) - (r[81 * s] * v[120 * s] * v[155 * s] * v[156 * s]) - (r[82 * s] * v[121 * s] * v[155 * s] * v[156 * s]) - (r[83 * s] * v[121 * s] * v[156 * s]) - (r[88 * s] * v[156 * s] * v[158 * s]) - (r[90 * s] * v[149 * s] * v[156 * s]) - (r[124 * s] * v[156 * s]) - (r[236 * s] * v[156 * s] * v[160 * s]) - (r[241 * s] * v[126 * s] * v[156 * s]) - (r[245 * s] * v[127 * s] * v[155 * s] * v[156 * s]) - (r[248 * s] * v[119 * s] * v[156 * s]) - (r[250 * s] * v[143 * s] * v[156 * s]) + (r[252 * s] * v[147 * s]) + (r[254 * s] * v[147 * s] * v[160 * s]);
    vdot[157 * s] = 0.0 + (r[5 * s] * v[88 * s]) - (r[21 * s] * v[157 * s]) - (r[69 * s] * v[144 * s] * v[157 * s]) - (r[70 * s] * v[156 * s] * v[157 * s]) - (r[71 * s] * v[157 * s] * v[159 * s]) - (r[86 * s] * v[150 * s] * v[157 * s]) - (r[92 * s] * v[151 * s] * v[157 * s]) - (r[100 * s] * v[157 * s]);
    vdot[158 * s] = 0.0 + (r[13 * s] * v[95 * s]) - (r[29 * s] * v[158 * s]) + -0x1.0000000000000p+1 * (r[87 * s] * v[144 * s] * v[158 * s]) + -0x1.0000000000000p+1 * (r[88 * s] * v[156 * s] * v[158 * s]) + -0x1.0000000000000p+1 * (r[89 * s] * v[158 * s] * v[159 * s]) + (r[93 * s] * v[151 * s] * v[160 * s]) + (r[94 * s] * v[125 * s] * v[160 * s]) - (r[132 * s] * v[158 * s]) + (r[231 * s] * v[146 * s]) - (r[237 * s] * v[154 * s] * v[158 * s]) - (r[238 * s] * v[150 * s] * v[158 * s]) + (r[239 * s] * v[149 * s]);
    vdot[159 * s] = 0.0 + (r[41 * s] * v[156 * s]) - (r[55 * s] * v[155 * s] * v[159 * s]) - (r[71 * s] * v[157 * s] * v[159 * s]) - (r[74 * s] * v[13 * s] * v[159 * s]) - (r[77 * s] * v[12 * s] * v[159 * s]) - (r[80 * s] * v[12 * s] * v[13 * s] * v[159 * s]) - (r[89 * s] * v[158 * s] * v[159 * s]) - (r[125 * s] * v[159 * s]) - (r[251 * s] * v[143 * s] * v[159 * s]) + (r[253 * s] * v[147 * s] * v[152 * s]);
}

KQ_HD KQ_NOINLINE void kqu_fun_9(const double* v, const double* f, const double* r, double* vdot, long long s)
{
    vdot[160 * s] = 0.0 + (r[86 * s] * v[150 * s] * v[157 * s]) - (r[93 * s] * v[151 * s] * v[160 * s]) - (r[94 * s] * v[125 * s] * v[160 * s]) + (r[137 * s] * f[1 * s]) - (r[138 * s] * v[160 * s]) - (r[139 * s] * v[160 * s]) + 0x1.0000000000000p+1 * (r[192 * s] * v[145 * s]) - (r[193 * s] * v[104 * s] * v[160 * s]) - (r[194 * s] * v[104 * s] * v[160 * s]) - (r[195 * s] * v[138 * s] * v[160 * s]) - (r[196 * s] * v[139 * s] * v[160 * s]) - (r[197 * s] * v[105 * s] * v[160 * s]) - (r[198 * s] * v[136 * s] * v[160 * s]) - (r[199 * s] * v[140 * s] * v[160 * s]) + -0x1.0000000000000p+1 * (r[200 * s] * v[128 * s] * v[160 * s]) - (r[201 * s] * v[131 * s] * v[160 * s]) - (r[202 * s] * v[130 * s] * v[160 * s]) - (r[203 * s] * v[112 * s] * v[160 * s]) - (r[204 * s] * v[133 * s] * v[160 * s]) - (r[205 * s] * v[132 * s] * v[160 * s]) - (r[206 * s] * v[134 * s] * v[160 * s]) - (r[207 * s] * v[135 * s] * v[160 * s]) - (r[208 * s] * v[148 * s] * v[160 * s]) - (r[209 * s] * v[141 * s] * v[160 * s]) + (r[231 * s] * v[146 * s]) + -0x1.0000000000000p+1 * (r[232 * s] * v[160 * s] * v[160 * s]) - (r[233 * s] * v[154 * s] * v[160 * s]) - (r[234 * s] * v[150 * s] * v[160 * s]) - (r[235 * s] * v[145 * s] * v[160 * s]) - (r[236 * s] * v[156 * s] * v[160 * s]) + (r[246 * s] * v[122 * s] * f[0 * s]) - (r[249 * s] * v[137 * s] * v[160 * s]) - (r[254 * s] * v[147 * s] * v[160 * s]);
}

KQ_HD inline void kqu_fun(const double* v, const double* f, const double* r, double* vdot, long long s)
{
    kqu_fun_0(v, f, r, vdot, s);
    kqu_fun_1(v, f, r, vdot, s);
    kqu_fun_2(v, f, r, vdot, s);
    kqu_fun_3(v, f, r, vdot, s);
    kqu_fun_4(v, f, r, vdot, s);
    kqu_fun_5(v, f, r, vdot, s);
    kqu_fun_6(v, f, r, vdot, s);
    kqu_fun_7(v, f, r, vdot, s);
    kqu_fun_8(v, f, r, vdot, s);
    kqu_fun_9(v, f, r, vdot, s);
}

KQ_HD KQ_NOINLINE void kqu_jac_0(const double* v, const double* f, const double* r, double* jvs, long long s)
{
    jvs[0 * s] = 0.0 - (r[32 * s]);
    jvs[1 * s] = 0.0 - (r[33 * s]);
    jvs[2 * s] = 0.0 - (r[34 * s]);
    jvs[3 * s] = 0.0 - (r[35 * s]);
    jvs[4 * s] = 0.0 - (r[36 * s]);
    jvs[5 * s] = 0.0 - (r[37 * s]);
    jvs[6 * s] = 0.0 - (r[38 * s]);
    jvs[7 * s] = 0.0 - (r[39 * s]);
    jvs[8 * s] = 0.0 + (r[39 * s]);
    jvs[9 * s] = 0.0 - (r[112 * s]);
    jvs[10 * s] = 0.0 + (r[37 * s]);
    jvs[11 * s] = 0.0 - (r[113 * s]);
    jvs[12 * s] = 0.0 - (r[114 * s]);
    jvs[13 * s] = 0.0 + (r[38 * s]);
    jvs[14 * s] = 0.0 - (r[115 * s]);
    jvs[15 * s] = 0.0 - (r[120 * s]);
    jvs[16 * s] = 0.0 - (r[121 * s]);
    jvs[17 * s] = 0.0 - (r[116 * s]);
    jvs[18 * s] = 0.0 - (r[117 * s]);
    jvs[19 * s] = 0.0 - (r[118 * s]);
    jvs[20 * s] = 0.0 + (r[35 * s]);
    jvs[21 * s] = 0.0 - (r[119 * s]);
    jvs[22 * s] = 0.0;
    jvs[23 * s] = 0.0 + (r[263 * s]);
    jvs[24 * s] = 0.0 + (r[262 * s]);
    jvs[25 * s] = 0.0 + (r[266 * s]);
    jvs[26 * s] = 0.0 + (r[265 * s]);
    jvs[27 * s] = 0.0 + (r[95 * s]);
    jvs[28 * s] = 0.0 + (r[264 * s]);
    jvs[29 * s] = 0.0 + (r[124 * s]);
    jvs[30 * s] = 0.0 + (r[125 * s]);
    jvs[31 * s] = 0.0;
    jvs[32 * s] = 0.0 + (r[96 * s]);
    jvs[33 * s] = 0.0;
    jvs[34 * s] = 0.0 + (r[267 * s]);
    jvs[35 * s] = 0.0 + (r[127 * s]);
    jvs[36 * s] = 0.0 + (r[126 * s]);
    jvs[37 * s] = 0.0 + (r[97 * s]);
    jvs[38 * s] = 0.0 - (r[267 * s]);
    jvs[39 * s] = 0.0 + (r[202 * s] * v[160 * s]);
    jvs[40 * s] = 0.0 + (r[201 * s] * v[160 * s]);
    jvs[41 * s] = 0.0 + (r[201 * s] * v[131 * s]) + (r[202 * s] * v[130 * s]);
    jvs[42 * s] = 0.0;
    jvs[43 * s] = 0.0 + (r[98 * s]);
    jvs[44 * s] = 0.0;
    jvs[45 * s] = 0.0 + (r[99 * s]);
    jvs[46 * s] = 0.0;
    jvs[47 * s] = 0.0 + (r[100 * s]);
    jvs[48 * s] = 0.0;
    jvs[49 * s] = 0.0 + (r[128 * s]);
    jvs[50 * s] = 0.0 + (r[101 * s]);
    jvs[51 * s] = 0.0;
    jvs[52 * s] = 0.0 + (r[102 * s]);
    jvs[53 * s] = 0.0;
    jvs[54 * s] = 0.0 + (r[103 * s]);
    jvs[55 * s] = 0.0;
    jvs[56 * s] = 0.0 + (r[104 * s]);
    jvs[57 * s] = 0.0 + (r[129 * s]);
    jvs[58 * s] = 0.0 + (r[108 * s]);
    jvs[59 * s] = 0.0;
    jvs[60 * s] = 0.0 + (r[105 * s]);
    jvs[61 * s] = 0.0;
    jvs[62 * s] = 0.0 + (r[106 * s]);
    jvs[63 * s] = 0.0;
    jvs[64 * s] = 0.0 + (r[107 * s]);
    jvs[65 * s] = 0.0;
    jvs[66 * s] = 0.0 + (r[139 * s]);
    jvs[67 * s] = 0.0;
    jvs[68 * s] = 0.0 + (r[109 * s]);
    jvs[69 * s] = 0.0;
    jvs[70 * s] = 0.0 + (r[110 * s]);
    jvs[71 * s] = 0.0;
    jvs[72 * s] = 0.0 + (r[111 * s]);
    jvs[73 * s] = 0.0 + (r[112 * s]);
    jvs[74 * s] = 0.0;
    jvs[75 * s] = 0.0 + (r[120 * s]);
    jvs[76 * s] = 0.0;
    jvs[77 * s] = 0.0 + (r[121 * s]);
    jvs[78 * s] = 0.0;
    jvs[79 * s] = 0.0 + (r[113 * s]);
    jvs[80 * s] = 0.0;
    jvs[81 * s] = 0.0 + (r[114 * s]);
    jvs[82 * s] = 0.0;
    jvs[83 * s] = 0.0 + (r[115 * s]);
    jvs[84 * s] = 0.0;
    jvs[85 * s] = 0.0;
    jvs[86 * s] = 0.0 + (r[122 * s]);
    jvs[87 * s] = 0.0 + (r[116 * s]);
    jvs[88 * s] = 0.0;
    jvs[89 * s] = 0.0 + (r[117 * s]);
    jvs[90 * s] = 0.0;
    jvs[91 * s] = 0.0 + (r[118 * s]);
    jvs[92 * s] = 0.0;
    jvs[93 * s] = 0.0 + (r[119 * s]);
    jvs[94 * s] = 0.0;
    jvs[95 * s] = 0.0;
    jvs[96 * s] = 0.0 + (r[132 * s]);
    jvs[97 * s] = 0.0;
    jvs[98 * s] = 0.0 + (r[133 * s]);
    jvs[99 * s] = 0.0 + (r[134 * s]);
    jvs[100 * s] = 0.0;
    jvs[101 * s] = 0.0 + (r[135 * s]);
    jvs[102 * s] = 0.0 + (r[136 * s]);
    jvs[103 * s] = 0.0;
    jvs[104 * s] = 0.0 + (r[157 * s]);
    jvs[105 * s] = 0.0;
    jvs[106 * s] = 0.0 + (r[165 * s]);
    jvs[107 * s] = 0.0 + (r[158 * s]);
    jvs[108 * s] = 0.0 - (r[165 * s]);
    jvs[109 * s] = 0.0 + (r[150 * s] * f[0 * s]) + (r[151 * s] * v[153 * s]) + (r[152 * s] * v[146 * s]);
    jvs[110 * s] = 0.0 + (r[152 * s] * v[115 * s]);
}

KQ_HD KQ_NOINLINE void kqu_jac_1(const double* v, const double* f, const double* r, double* jvs, long long s)
{
    jvs[111 * s] = 0.0 + (r[151 * s] * v[115 * s]);
    jvs[112 * s] = 0.0;
    jvs[113 * s] = 0.0 + (r[159 * s]);
    jvs[114 * s] = 0.0;
    jvs[115 * s] = 0.0 + (r[160 * s]);
    jvs[116 * s] = 0.0 - (r[160 * s]);
    jvs[117 * s] = 0.0 + (r[148 * s] * v[115 * s]);
    jvs[118 * s] = 0.0 + (r[149 * s] * v[115 * s]);
    jvs[119 * s] = 0.0 + (r[148 * s] * v[101 * s]) + (r[149 * s] * v[102 * s]);
    jvs[120 * s] = 0.0;
    jvs[121 * s] = 0.0 + (r[161 * s]);
    jvs[122 * s] = 0.0;
    jvs[123 * s] = 0.0 + (r[162 * s]);
    jvs[124 * s] = 0.0;
    jvs[125 * s] = 0.0 + (r[163 * s]);
    jvs[126 * s] = 0.0 - (r[163 * s]);
    jvs[127 * s] = 0.0 + (r[153 * s] * f[0 * s]);
    jvs[128 * s] = 0.0 + (r[155 * s] * f[0 * s]);
    jvs[129 * s] = 0.0;
    jvs[130 * s] = 0.0 + (r[164 * s]);
    jvs[131 * s] = 0.0 - (r[164 * s]);
    jvs[132 * s] = 0.0 + (r[154 * s] * v[153 * s]);
    jvs[133 * s] = 0.0 + (r[156 * s] * v[153 * s]);
    jvs[134 * s] = 0.0 + (r[154 * s] * v[75 * s]) + (r[156 * s] * v[77 * s]);
    jvs[135 * s] = 0.0;
    jvs[136 * s] = 0.0 + (r[211 * s]);
    jvs[137 * s] = 0.0 + (r[212 * s]);
    jvs[138 * s] = 0.0;
    jvs[139 * s] = 0.0 + (r[213 * s]);
    jvs[140 * s] = 0.0 + (r[215 * s]);
    jvs[141 * s] = 0.0 + (r[214 * s]);
    jvs[142 * s] = 0.0;
    jvs[143 * s] = 0.0 + (r[217 * s]);
    jvs[144 * s] = 0.0 + (r[216 * s]);
    jvs[145 * s] = 0.0;
    jvs[146 * s] = 0.0 + (r[218 * s]);
    jvs[147 * s] = 0.0 + (r[219 * s]);
    jvs[148 * s] = 0.0;
    jvs[149 * s] = 0.0 + (r[224 * s]);
    jvs[150 * s] = 0.0 + (r[264 * s]);
    jvs[151 * s] = 0.0 + (r[220 * s]);
    jvs[152 * s] = 0.0;
    jvs[153 * s] = 0.0 + (r[130 * s]);
    jvs[154 * s] = 0.0 + (r[131 * s]);
    jvs[155 * s] = 0.0;
    jvs[156 * s] = 0.0 + (r[221 * s]);
    jvs[157 * s] = 0.0;
    jvs[158 * s] = 0.0 + (r[222 * s]);
    jvs[159 * s] = 0.0 + (r[223 * s]);
    jvs[160 * s] = 0.0;
    jvs[161 * s] = 0.0 + (r[226 * s]);
    jvs[162 * s] = 0.0 + (r[268 * s]);
    jvs[163 * s] = 0.0 + (r[225 * s]);
    jvs[164 * s] = 0.0;
    jvs[165 * s] = 0.0 + (r[260 * s]);
    jvs[166 * s] = 0.0;
    jvs[167 * s] = 0.0 + (r[261 * s]);
    jvs[168 * s] = 0.0 - (r[14 * s]);
    jvs[169 * s] = 0.0 + (r[30 * s]);
    jvs[170 * s] = 0.0 - (r[141 * s]);
    jvs[171 * s] = 0.0 + (r[144 * s]);
    jvs[172 * s] = 0.0 + (r[141 * s]);
    jvs[173 * s] = 0.0 - (r[144 * s]) - (r[153 * s] * f[0 * s]) - (r[154 * s] * v[153 * s]) - (r[161 * s]);
    jvs[174 * s] = 0.0 - (r[154 * s] * v[75 * s]);
    jvs[175 * s] = 0.0 - (r[142 * s]);
    jvs[176 * s] = 0.0 + (r[145 * s]);
    jvs[177 * s] = 0.0 + (r[142 * s]);
    jvs[178 * s] = 0.0 - (r[145 * s]) - (r[155 * s] * f[0 * s]) - (r[156 * s] * v[153 * s]) - (r[162 * s]);
    jvs[179 * s] = 0.0 - (r[156 * s] * v[77 * s]);
    jvs[180 * s] = 0.0 - (r[166 * s]);
    jvs[181 * s] = 0.0 + (r[171 * s]);
    jvs[182 * s] = 0.0 - (r[167 * s]);
    jvs[183 * s] = 0.0 + (r[172 * s]);
    jvs[184 * s] = 0.0 - (r[168 * s]);
    jvs[185 * s] = 0.0 + (r[173 * s]);
    jvs[186 * s] = 0.0 - (r[12 * s]);
    jvs[187 * s] = 0.0 + (r[28 * s]);
    jvs[188 * s] = 0.0 - (r[170 * s]);
    jvs[189 * s] = 0.0 + (r[175 * s]);
    jvs[190 * s] = 0.0 - (r[169 * s]);
    jvs[191 * s] = 0.0 + (r[174 * s]);
    jvs[192 * s] = 0.0 - (r[4 * s]);
    jvs[193 * s] = 0.0 + (r[20 * s]);
    jvs[194 * s] = 0.0 - (r[1 * s]);
    jvs[195 * s] = 0.0 + (r[17 * s]);
    jvs[196 * s] = 0.0 - (r[2 * s]);
    jvs[197 * s] = 0.0 + (r[18 * s]);
    jvs[198 * s] = 0.0 - (r[3 * s]);
    jvs[199 * s] = 0.0 + (r[19 * s]);
    jvs[200 * s] = 0.0 - (r[5 * s]);
    jvs[201 * s] = 0.0 + (r[21 * s]);
    jvs[202 * s] = 0.0 - (r[6 * s]);
    jvs[203 * s] = 0.0 + (r[22 * s]);
    jvs[204 * s] = 0.0 - (r[7 * s]);
    jvs[205 * s] = 0.0 + (r[23 * s]);
    jvs[206 * s] = 0.0 - (r[8 * s]);
}

KQ_HD KQ_NOINLINE void kqu_jac_2(const double* v, const double* f, const double* r, double* jvs, long long s)
{
    jvs[207 * s] = 0.0 + (r[24 * s]);
    jvs[208 * s] = 0.0 - (r[9 * s]);
    jvs[209 * s] = 0.0 + (r[25 * s]);
    jvs[210 * s] = 0.0 - (r[10 * s]);
    jvs[211 * s] = 0.0 + (r[26 * s]);
    jvs[212 * s] = 0.0 - (r[11 * s]);
    jvs[213 * s] = 0.0 + (r[27 * s]);
    jvs[214 * s] = 0.0 - (r[13 * s]);
    jvs[215 * s] = 0.0 + (r[29 * s]);
    jvs[216 * s] = 0.0 - (r[15 * s]);
    jvs[217 * s] = 0.0 + (r[31 * s]);
    jvs[218 * s] = 0.0 - (r[227 * s]);
    jvs[219 * s] = 0.0 + (r[229 * s]);
    jvs[220 * s] = 0.0 - (r[228 * s]);
    jvs[221 * s] = 0.0 + (r[230 * s]);
    jvs[222 * s] = 0.0 - (r[0 * s]);
    jvs[223 * s] = 0.0 + (r[16 * s]);
    jvs[224 * s] = 0.0 - (r[140 * s]);
    jvs[225 * s] = 0.0 + (r[143 * s]);
    jvs[226 * s] = 0.0 - (r[148 * s] * v[115 * s]) - (r[158 * s]);
    jvs[227 * s] = 0.0 + (r[146 * s] * f[0 * s]) - (r[148 * s] * v[101 * s]);
    jvs[228 * s] = 0.0 - (r[149 * s] * v[115 * s]) - (r[159 * s]);
    jvs[229 * s] = 0.0 + (r[147 * s] * v[153 * s]) - (r[149 * s] * v[102 * s]);
    jvs[230 * s] = 0.0 + (r[147 * s] * v[115 * s]);
    jvs[231 * s] = 0.0 - (r[242 * s] * f[2 * s]) - (r[263 * s]);
    jvs[232 * s] = 0.0 + (r[248 * s] * v[156 * s]);
    jvs[233 * s] = 0.0 + (r[241 * s] * v[156 * s]);
    jvs[234 * s] = 0.0 + (r[236 * s] * v[160 * s]) + (r[241 * s] * v[126 * s]) + (r[248 * s] * v[119 * s]);
    jvs[235 * s] = 0.0 + (r[236 * s] * v[156 * s]);
    jvs[236 * s] = 0.0 + (r[166 * s]);
    jvs[237 * s] = 0.0 - (r[171 * s]) - (r[193 * s] * v[160 * s]) - (r[194 * s] * v[160 * s]) - (r[221 * s]);
    jvs[238 * s] = 0.0 - (r[193 * s] * v[104 * s]) - (r[194 * s] * v[104 * s]);
    jvs[239 * s] = 0.0 + (r[10 * s]);
    jvs[240 * s] = 0.0 + (r[194 * s] * v[160 * s]);
    jvs[241 * s] = 0.0 - (r[26 * s]) - (r[106 * s]) - (r[197 * s] * v[160 * s]);
    jvs[242 * s] = 0.0 + (r[194 * s] * v[104 * s]) - (r[197 * s] * v[105 * s]);
    jvs[243 * s] = 0.0 + (r[1 * s]);
    jvs[244 * s] = 0.0 - (r[17 * s]) - (r[42 * s]) - (r[96 * s]);
    jvs[245 * s] = 0.0 + (r[56 * s] * v[155 * s]);
    jvs[246 * s] = 0.0 + (r[56 * s] * v[146 * s]);
    jvs[247 * s] = 0.0 + (r[3 * s]);
    jvs[248 * s] = 0.0 - (r[19 * s]) - (r[45 * s]) - (r[98 * s]);
    jvs[249 * s] = 0.0 + (r[59 * s] * v[152 * s]);
    jvs[250 * s] = 0.0 + (r[59 * s] * v[108 * s]);
    jvs[251 * s] = 0.0 + (r[33 * s]);
    jvs[252 * s] = 0.0 + (r[45 * s]);
    jvs[253 * s] = 0.0 - (r[59 * s] * v[152 * s]) - (r[110 * s]);
    jvs[254 * s] = 0.0 - (r[59 * s] * v[108 * s]);
    jvs[255 * s] = 0.0 - (r[49 * s]) - (r[104 * s]);
    jvs[256 * s] = 0.0 + (r[63 * s] * v[155 * s]);
    jvs[257 * s] = 0.0 + (r[63 * s] * v[123 * s]);
    jvs[258 * s] = 0.0 + (r[9 * s]);
    jvs[259 * s] = 0.0 - (r[25 * s]) - (r[47 * s]) - (r[105 * s]);
    jvs[260 * s] = 0.0 + (r[61 * s] * v[155 * s]);
    jvs[261 * s] = 0.0 + (r[61 * s] * v[111 * s]);
    jvs[262 * s] = 0.0 + (r[34 * s]);
    jvs[263 * s] = 0.0 + (r[47 * s]);
    jvs[264 * s] = 0.0 - (r[61 * s] * v[155 * s]) - (r[111 * s]);
    jvs[265 * s] = 0.0 - (r[61 * s] * v[111 * s]);
    jvs[266 * s] = 0.0 + (r[11 * s]);
    jvs[267 * s] = 0.0 - (r[27 * s]) - (r[107 * s]) - (r[203 * s] * v[160 * s]);
    jvs[268 * s] = 0.0 - (r[203 * s] * v[112 * s]);
    jvs[269 * s] = 0.0 - (r[58 * s] * v[155 * s]) - (r[127 * s]);
    jvs[270 * s] = 0.0 + (r[44 * s]);
    jvs[271 * s] = 0.0 - (r[58 * s] * v[113 * s]);
    jvs[272 * s] = 0.0 + (r[58 * s] * v[155 * s]);
}

KQ_HD KQ_NOINLINE void kqu_jac_3(const double* v, const double* f, const double* r, double* jvs, long long s)
{
    jvs[273 * s] = 0.0 - (r[44 * s]) - (r[57 * s] * v[155 * s]) - (r[126 * s]);
    jvs[274 * s] = 0.0 + (r[43 * s]);
    jvs[275 * s] = 0.0 - (r[57 * s] * v[114 * s]) + (r[58 * s] * v[113 * s]);
    jvs[276 * s] = 0.0 + (r[140 * s]);
    jvs[277 * s] = 0.0 - (r[148 * s] * v[115 * s]);
    jvs[278 * s] = 0.0 - (r[149 * s] * v[115 * s]);
    jvs[279 * s] = 0.0 - (r[143 * s]) - (r[146 * s] * f[0 * s]) - (r[147 * s] * v[153 * s]) - (r[148 * s] * v[101 * s]) - (r[149 * s] * v[102 * s]) - (r[150 * s] * f[0 * s]) - (r[151 * s] * v[153 * s]) - (r[152 * s] * v[146 * s]) - (r[157 * s]);
    jvs[280 * s] = 0.0 - (r[152 * s] * v[115 * s]);
    jvs[281 * s] = 0.0 - (r[147 * s] * v[115 * s]) - (r[151 * s] * v[115 * s]);
    jvs[282 * s] = 0.0 - (r[191 * s]) - (r[210 * s] * v[160 * s]) - (r[226 * s]);
    jvs[283 * s] = 0.0 + (r[258 * s] * v[152 * s]);
    jvs[284 * s] = 0.0 + (r[190 * s] * f[0 * s]);
    jvs[285 * s] = 0.0 + (r[258 * s] * v[117 * s]);
    jvs[286 * s] = 0.0 - (r[210 * s] * v[116 * s]);
    jvs[287 * s] = 0.0 - (r[257 * s]) - (r[258 * s] * v[152 * s]) - (r[259 * s] * v[160 * s]) - (r[268 * s]);
    jvs[288 * s] = 0.0 + (r[255 * s] * v[156 * s]) + (r[256 * s] * v[159 * s]);
    jvs[289 * s] = 0.0 - (r[258 * s] * v[117 * s]);
    jvs[290 * s] = 0.0 + (r[255 * s] * v[118 * s]);
    jvs[291 * s] = 0.0 + (r[256 * s] * v[118 * s]);
    jvs[292 * s] = 0.0 - (r[259 * s] * v[117 * s]);
    jvs[293 * s] = 0.0 + (r[169 * s]);
    jvs[294 * s] = 0.0 + (r[191 * s]);
    jvs[295 * s] = 0.0 + (r[257 * s]);
    jvs[296 * s] = 0.0 - (r[174 * s]) - (r[190 * s] * f[0 * s]) - (r[225 * s]) - (r[255 * s] * v[156 * s]) - (r[256 * s] * v[159 * s]);
    jvs[297 * s] = 0.0;
    jvs[298 * s] = 0.0 - (r[255 * s] * v[118 * s]);
    jvs[299 * s] = 0.0 - (r[256 * s] * v[118 * s]);
    jvs[300 * s] = 0.0;
    jvs[301 * s] = 0.0 + (r[228 * s]);
    jvs[302 * s] = 0.0 - (r[230 * s]) + -0x1.0000000000000p+1 * (r[247 * s] * 0x1.0000000000000p+1 * v[119 * s]) - (r[248 * s] * v[156 * s]) - (r[261 * s]);
    jvs[303 * s] = 0.0 - (r[248 * s] * v[119 * s]);
    jvs[304 * s] = 0.0 + (r[7 * s]);
    jvs[305 * s] = 0.0 + (r[248 * s] * v[156 * s]);
    jvs[306 * s] = 0.0 - (r[23 * s]) - (r[81 * s] * v[155 * s] * v[156 * s]) - (r[102 * s]);
    jvs[307 * s] = 0.0 - (r[81 * s] * v[120 * s] * v[156 * s]);
    jvs[308 * s] = 0.0 - (r[81 * s] * v[120 * s] * v[155 * s]) + (r[248 * s] * v[119 * s]);
    jvs[309 * s] = 0.0 + (r[8 * s]);
    jvs[310 * s] = 0.0 - (r[24 * s]) - (r[82 * s] * v[155 * s] * v[156 * s]) - (r[83 * s] * v[156 * s]) - (r[103 * s]);
    jvs[311 * s] = 0.0 - (r[82 * s] * v[121 * s] * v[156 * s]);
    jvs[312 * s] = 0.0 - (r[82 * s] * v[121 * s] * v[155 * s]) - (r[83 * s] * v[121 * s]);
    jvs[313 * s] = 0.0 - (r[246 * s] * f[0 * s]) - (r[262 * s]);
    jvs[314 * s] = 0.0 + (r[240 * s] * v[153 * s]);
    jvs[315 * s] = 0.0 + 0x1.0000000000000p+1 * (r[244 * s] * 0x1.0000000000000p+1 * v[142 * s]);
    jvs[316 * s] = 0.0 + (r[240 * s] * v[126 * s]);
    jvs[317 * s] = 0.0 + (r[49 * s]);
    jvs[318 * s] = 0.0 + (r[246 * s] * f[0 * s]);
    jvs[319 * s] = 0.0 - (r[50 * s]) - (r[63 * s] * v[155 * s]) - (r[129 * s]);
    jvs[320 * s] = 0.0;
    jvs[321 * s] = 0.0;
    jvs[322 * s] = 0.0 + (r[64 * s] * v[155 * s]);
    jvs[323 * s] = 0.0 - (r[63 * s] * v[123 * s]) + (r[64 * s] * v[153 * s]);
    jvs[324 * s] = 0.0 + (r[2 * s]);
    jvs[325 * s] = 0.0 + (r[57 * s] * v[155 * s]);
}

KQ_HD KQ_NOINLINE void kqu_jac_4(const double* v, const double* f, const double* r, double* jvs, long long s)
{
    jvs[326 * s] = 0.0 - (r[18 * s]) - (r[43 * s]) - (r[97 * s]);
    jvs[327 * s] = 0.0 + 0x1.0000000000000p+1 * (r[200 * s] * v[160 * s]);
    jvs[328 * s] = 0.0 + (r[202 * s] * v[160 * s]);
    jvs[329 * s] = 0.0 + (r[201 * s] * v[160 * s]);
    jvs[330 * s] = 0.0 + (r[205 * s] * v[160 * s]);
    jvs[331 * s] = 0.0 + (r[204 * s] * v[160 * s]);
    jvs[332 * s] = 0.0 + (r[249 * s] * v[160 * s]);
    jvs[333 * s] = 0.0 + (r[209 * s] * v[160 * s]);
    jvs[334 * s] = 0.0 + (r[57 * s] * v[114 * s]);
    jvs[335 * s] = 0.0 + 0x1.0000000000000p+1 * (r[200 * s] * v[128 * s]) + (r[201 * s] * v[131 * s]) + (r[202 * s] * v[130 * s]) + (r[204 * s] * v[133 * s]) + (r[205 * s] * v[132 * s]) + (r[209 * s] * v[141 * s]) + (r[249 * s] * v[137 * s]);
    jvs[336 * s] = 0.0 + (r[14 * s]);
    jvs[337 * s] = 0.0 - (r[30 * s]) - (r[52 * s]) - (r[94 * s] * v[160 * s]) - (r[133 * s]);
    jvs[338 * s] = 0.0 + (r[66 * s] * v[155 * s]);
    jvs[339 * s] = 0.0 + (r[66 * s] * v[151 * s]);
    jvs[340 * s] = 0.0 - (r[94 * s] * v[125 * s]);
    jvs[341 * s] = 0.0 + (r[227 * s]);
    jvs[342 * s] = 0.0 - (r[229 * s]) - (r[240 * s] * v[153 * s]) - (r[241 * s] * v[156 * s]) - (r[260 * s]);
    jvs[343 * s] = 0.0 - (r[240 * s] * v[126 * s]);
    jvs[344 * s] = 0.0 - (r[241 * s] * v[126 * s]);
    jvs[345 * s] = 0.0 - (r[245 * s] * v[155 * s] * v[156 * s]) - (r[266 * s]);
    jvs[346 * s] = 0.0 + (r[243 * s] * v[154 * s]);
    jvs[347 * s] = 0.0 + (r[243 * s] * v[142 * s]);
    jvs[348 * s] = 0.0 - (r[245 * s] * v[127 * s] * v[156 * s]);
    jvs[349 * s] = 0.0 - (r[245 * s] * v[127 * s] * v[155 * s]);
    jvs[350 * s] = 0.0 - (r[177 * s]) - (r[200 * s] * v[160 * s]) - (r[213 * s]);
    jvs[351 * s] = 0.0 + (r[183 * s] * v[155 * s]);
    jvs[352 * s] = 0.0 + (r[198 * s] * v[160 * s]);
    jvs[353 * s] = 0.0 + (r[183 * s] * v[131 * s]);
    jvs[354 * s] = 0.0 + (r[198 * s] * v[136 * s]) - (r[200 * s] * v[128 * s]);
    jvs[355 * s] = 0.0 - (r[67 * s] * v[155 * s]) - (r[91 * s]) - (r[135 * s]);
    jvs[356 * s] = 0.0 + (r[53 * s]);
    jvs[357 * s] = 0.0 + (r[238 * s] * v[158 * s]);
    jvs[358 * s] = 0.0 - (r[67 * s] * v[129 * s]);
    jvs[359 * s] = 0.0 + (r[238 * s] * v[150 * s]);
    jvs[360 * s] = 0.0 - (r[184 * s] * v[155 * s]) - (r[202 * s] * v[160 * s]) - (r[215 * s]);
    jvs[361 * s] = 0.0 + (r[178 * s]);
    jvs[362 * s] = 0.0 - (r[184 * s] * v[130 * s]);
    jvs[363 * s] = 0.0 - (r[202 * s] * v[130 * s]);
    jvs[364 * s] = 0.0 + (r[177 * s]);
    jvs[365 * s] = 0.0 + (r[184 * s] * v[155 * s]);
    jvs[366 * s] = 0.0 - (r[178 * s]) - (r[183 * s] * v[155 * s]) - (r[201 * s] * v[160 * s]) - (r[214 * s]);
    jvs[367 * s] = 0.0;
    jvs[368 * s] = 0.0 + (r[199 * s] * v[160 * s]);
    jvs[369 * s] = 0.0 - (r[183 * s] * v[131 * s]) + (r[184 * s] * v[130 * s]);
    jvs[370 * s] = 0.0 + (r[199 * s] * v[140 * s]) - (r[201 * s] * v[131 * s]);
    jvs[371 * s] = 0.0 + 0x1.d70a3e0000000p-1 * (r[203 * s] * v[160 * s]);
    jvs[372 * s] = 0.0 - (r[185 * s] * v[155 * s]) - (r[205 * s] * v[160 * s]) - (r[217 * s]);
    jvs[373 * s] = 0.0 + (r[179 * s]);
    jvs[374 * s] = 0.0 - (r[185 * s] * v[132 * s]);
    jvs[375 * s] = 0.0 + 0x1.d70a3e0000000p-1 * (r[203 * s] * v[112 * s]) - (r[205 * s] * v[132 * s]);
    jvs[376 * s] = 0.0 + (r[170 * s]);
    jvs[377 * s] = 0.0 + (r[185 * s] * v[155 * s]);
    jvs[378 * s] = 0.0 - (r[175 * s]) - (r[179 * s]) - (r[204 * s] * v[160 * s]) - (r[216 * s]);
}

KQ_HD KQ_NOINLINE void kqu_jac_5(const double* v, const double* f, const double* r, double* jvs, long long s)
{
    jvs[379 * s] = 0.0 + (r[185 * s] * v[132 * s]);
    jvs[380 * s] = 0.0 - (r[204 * s] * v[133 * s]);
    jvs[381 * s] = 0.0 + (r[167 * s]);
    jvs[382 * s] = 0.0 + (r[204 * s] * v[160 * s]);
    jvs[383 * s] = 0.0 - (r[172 * s]) - (r[181 * s]) - (r[206 * s] * v[160 * s]) - (r[218 * s]);
    jvs[384 * s] = 0.0 + (r[187 * s] * v[155 * s]);
    jvs[385 * s] = 0.0 + (r[187 * s] * v[135 * s]);
    jvs[386 * s] = 0.0 + (r[204 * s] * v[133 * s]) - (r[206 * s] * v[134 * s]);
    jvs[387 * s] = 0.0 + (r[205 * s] * v[160 * s]);
    jvs[388 * s] = 0.0;
    jvs[389 * s] = 0.0 + (r[181 * s]);
    jvs[390 * s] = 0.0 - (r[187 * s] * v[155 * s]) - (r[207 * s] * v[160 * s]) - (r[219 * s]);
    jvs[391 * s] = 0.0 - (r[187 * s] * v[135 * s]);
    jvs[392 * s] = 0.0 + (r[205 * s] * v[132 * s]) - (r[207 * s] * v[135 * s]);
    jvs[393 * s] = 0.0 + (r[197 * s] * v[160 * s]);
    jvs[394 * s] = 0.0 + 0x1.b333340000000p-1 * (r[206 * s] * v[160 * s]);
    jvs[395 * s] = 0.0;
    jvs[396 * s] = 0.0 - (r[176 * s]) - (r[198 * s] * v[160 * s]) - (r[211 * s]);
    jvs[397 * s] = 0.0 + (r[182 * s] * v[155 * s]);
    jvs[398 * s] = 0.0 + (r[182 * s] * v[140 * s]);
    jvs[399 * s] = 0.0 + (r[197 * s] * v[105 * s]) - (r[198 * s] * v[136 * s]) + 0x1.b333340000000p-1 * (r[206 * s] * v[134 * s]);
    jvs[400 * s] = 0.0 - (r[60 * s] * v[155 * s]) - (r[128 * s]) - (r[249 * s] * v[160 * s]);
    jvs[401 * s] = 0.0 + (r[46 * s]);
    jvs[402 * s] = 0.0 - (r[60 * s] * v[137 * s]);
    jvs[403 * s] = 0.0 - (r[249 * s] * v[137 * s]);
    jvs[404 * s] = 0.0 + (r[193 * s] * v[160 * s]);
    jvs[405 * s] = 0.0 - (r[180 * s]) - (r[195 * s] * v[160 * s]) - (r[222 * s]);
    jvs[406 * s] = 0.0 + (r[186 * s] * v[155 * s]);
    jvs[407 * s] = 0.0 + (r[186 * s] * v[139 * s]);
    jvs[408 * s] = 0.0 + (r[193 * s] * v[104 * s]) - (r[195 * s] * v[138 * s]);
    jvs[409 * s] = 0.0 + (r[180 * s]);
    jvs[410 * s] = 0.0 - (r[186 * s] * v[155 * s]) - (r[196 * s] * v[160 * s]) - (r[223 * s]);
    jvs[411 * s] = 0.0 - (r[186 * s] * v[139 * s]);
    jvs[412 * s] = 0.0 - (r[196 * s] * v[139 * s]);
    jvs[413 * s] = 0.0 + 0x1.47ae140000000p-4 * (r[203 * s] * v[160 * s]);
    jvs[414 * s] = 0.0 + 0x1.b333340000000p-1 * (r[207 * s] * v[160 * s]);
    jvs[415 * s] = 0.0 + (r[176 * s]);
    jvs[416 * s] = 0.0 + (r[195 * s] * v[160 * s]);
    jvs[417 * s] = 0.0 + (r[196 * s] * v[160 * s]);
    jvs[418 * s] = 0.0 - (r[182 * s] * v[155 * s]) - (r[199 * s] * v[160 * s]) - (r[212 * s]);
    jvs[419 * s] = 0.0 - (r[182 * s] * v[140 * s]);
    jvs[420 * s] = 0.0 + (r[195 * s] * v[138 * s]) + (r[196 * s] * v[139 * s]) - (r[199 * s] * v[140 * s]) + 0x1.47ae140000000p-4 * (r[203 * s] * v[112 * s]) + 0x1.b333340000000p-1 * (r[207 * s] * v[135 * s]);
    jvs[421 * s] = 0.0 + (r[6 * s]);
    jvs[422 * s] = 0.0 + (r[60 * s] * v[155 * s]);
    jvs[423 * s] = 0.0 - (r[22 * s]) - (r[46 * s]) - (r[101 * s]) - (r[209 * s] * v[160 * s]);
    jvs[424 * s] = 0.0 + (r[254 * s] * v[160 * s]);
    jvs[425 * s] = 0.0 + (r[208 * s] * v[160 * s]);
    jvs[426 * s] = 0.0 + (r[60 * s] * v[137 * s]);
    jvs[427 * s] = 0.0 + (r[208 * s] * v[148 * s]) - (r[209 * s] * v[141 * s]) + (r[254 * s] * v[147 * s]);
    jvs[428 * s] = 0.0 + (r[242 * s] * f[2 * s]);
    jvs[429 * s] = 0.0;
    jvs[430 * s] = 0.0;
    jvs[431 * s] = 0.0 - (r[243 * s] * v[154 * s]) + -0x1.0000000000000p+1 * (r[244 * s] * 0x1.0000000000000p+1 * v[142 * s]) - (r[265 * s]);
    jvs[432 * s] = 0.0;
    jvs[433 * s] = 0.0 - (r[243 * s] * v[142 * s]);
    jvs[434 * s] = 0.0;
    jvs[435 * s] = 0.0;
    jvs[436 * s] = 0.0 + (r[168 * s]);
}

KQ_HD KQ_NOINLINE void kqu_jac_6(const double* v, const double* f, const double* r, double* jvs, long long s)
{
    jvs[437 * s] = 0.0 + 0x1.0000000000000p+1 * (r[247 * s] * 0x1.0000000000000p+1 * v[119 * s]);
    jvs[438 * s] = 0.0 - (r[173 * s]) - (r[188 * s] * f[0 * s]) - (r[224 * s]) - (r[250 * s] * v[156 * s]) - (r[251 * s] * v[159 * s]);
    jvs[439 * s] = 0.0 + (r[252 * s]);
    jvs[440 * s] = 0.0 + (r[189 * s]);
    jvs[441 * s] = 0.0 - (r[250 * s] * v[143 * s]);
    jvs[442 * s] = 0.0 - (r[251 * s] * v[143 * s]);
    jvs[443 * s] = 0.0 - (r[75 * s] * v[144 * s]) - (r[78 * s] * v[13 * s] * v[144 * s]);
    jvs[444 * s] = 0.0 - (r[72 * s] * v[144 * s]) - (r[78 * s] * v[12 * s] * v[144 * s]);
    jvs[445 * s] = 0.0 + (r[0 * s]);
    jvs[446 * s] = 0.0 - (r[16 * s]) - (r[40 * s]) - (r[69 * s] * v[157 * s]) - (r[72 * s] * v[13 * s]) - (r[75 * s] * v[12 * s]) - (r[78 * s] * v[12 * s] * v[13 * s]) - (r[87 * s] * v[158 * s]) - (r[95 * s]);
    jvs[447 * s] = 0.0 + (r[54 * s] * v[156 * s]);
    jvs[448 * s] = 0.0 + (r[54 * s] * v[155 * s]);
    jvs[449 * s] = 0.0 - (r[69 * s] * v[144 * s]);
    jvs[450 * s] = 0.0 - (r[87 * s] * v[144 * s]);
    jvs[451 * s] = 0.0 + (r[4 * s]);
    jvs[452 * s] = 0.0 - (r[20 * s]) - (r[68 * s] * v[155 * s] * v[156 * s]) - (r[99 * s]) - (r[192 * s]) - (r[235 * s] * v[160 * s]);
    jvs[453 * s] = 0.0 + (r[85 * s] * v[154 * s]);
    jvs[454 * s] = 0.0 + (r[84 * s] * 0x1.0000000000000p+1 * v[154 * s]) + (r[85 * s] * v[150 * s]);
    jvs[455 * s] = 0.0 - (r[68 * s] * v[145 * s] * v[156 * s]);
    jvs[456 * s] = 0.0 - (r[68 * s] * v[145 * s] * v[155 * s]);
    jvs[457 * s] = 0.0 + (r[232 * s] * 0x1.0000000000000p+1 * v[160 * s]) - (r[235 * s] * v[145 * s]);
    jvs[458 * s] = 0.0 + (r[32 * s]);
    jvs[459 * s] = 0.0 + (r[42 * s]);
    jvs[460 * s] = 0.0 - (r[152 * s] * v[146 * s]);
    jvs[461 * s] = 0.0 + (r[240 * s] * v[153 * s]) + (r[241 * s] * v[156 * s]);
    jvs[462 * s] = 0.0 - (r[56 * s] * v[155 * s]) - (r[109 * s]) - (r[152 * s] * v[115 * s]) - (r[231 * s]);
    jvs[463 * s] = 0.0 + (r[90 * s] * v[156 * s]);
    jvs[464 * s] = 0.0 + (r[92 * s] * v[157 * s]);
    jvs[465 * s] = 0.0 + (r[240 * s] * v[126 * s]);
    jvs[466 * s] = 0.0 - (r[56 * s] * v[146 * s]);
    jvs[467 * s] = 0.0 + (r[90 * s] * v[149 * s]) + (r[241 * s] * v[126 * s]);
    jvs[468 * s] = 0.0 + (r[92 * s] * v[151 * s]);
    jvs[469 * s] = 0.0 + (r[250 * s] * v[156 * s]) + (r[251 * s] * v[159 * s]);
    jvs[470 * s] = 0.0 - (r[252 * s]) - (r[253 * s] * v[152 * s]) - (r[254 * s] * v[160 * s]) - (r[264 * s]);
    jvs[471 * s] = 0.0;
    jvs[472 * s] = 0.0 - (r[253 * s] * v[147 * s]);
    jvs[473 * s] = 0.0 + (r[250 * s] * v[143 * s]);
    jvs[474 * s] = 0.0 + (r[251 * s] * v[143 * s]);
    jvs[475 * s] = 0.0 - (r[254 * s] * v[147 * s]);
    jvs[476 * s] = 0.0 + 0x1.3333340000000p-3 * (r[206 * s] * v[160 * s]);
    jvs[477 * s] = 0.0 + 0x1.3333340000000p-3 * (r[207 * s] * v[160 * s]);
    jvs[478 * s] = 0.0 + (r[188 * s] * f[0 * s]);
    jvs[479 * s] = 0.0 + (r[253 * s] * v[152 * s]);
    jvs[480 * s] = 0.0 - (r[189 * s]) - (r[208 * s] * v[160 * s]) - (r[220 * s]);
    jvs[481 * s] = 0.0 + (r[253 * s] * v[147 * s]);
    jvs[482 * s] = 0.0;
    jvs[483 * s] = 0.0;
    jvs[484 * s] = 0.0;
    jvs[485 * s] = 0.0 + 0x1.3333340000000p-3 * (r[206 * s] * v[134 * s]) + 0x1.3333340000000p-3 * (r[207 * s] * v[135 * s]) - (r[208 * s] * v[148 * s]);
    jvs[486 * s] = 0.0 + (r[15 * s]);
    jvs[487 * s] = 0.0 + (r[67 * s] * v[155 * s]);
}

KQ_HD KQ_NOINLINE void kqu_jac_7(const double* v, const double* f, const double* r, double* jvs, long long s)
{
    jvs[488 * s] = 0.0 - (r[31 * s]) - (r[53 * s]) - (r[90 * s] * v[156 * s]) - (r[136 * s]) - (r[239 * s]);
    jvs[489 * s] = 0.0;
    jvs[490 * s] = 0.0 + (r[237 * s] * v[158 * s]);
    jvs[491 * s] = 0.0 + (r[67 * s] * v[129 * s]);
    jvs[492 * s] = 0.0 - (r[90 * s] * v[149 * s]);
    jvs[493 * s] = 0.0 + (r[237 * s] * v[154 * s]);
    jvs[494 * s] = 0.0 - (r[65 * s] * v[155 * s]) - (r[85 * s] * v[154 * s]) - (r[86 * s] * v[157 * s]) - (r[130 * s]) - (r[234 * s] * v[160 * s]) - (r[238 * s] * v[158 * s]);
    jvs[495 * s] = 0.0 + (r[51 * s]) - (r[85 * s] * v[150 * s]);
    jvs[496 * s] = 0.0 - (r[65 * s] * v[150 * s]);
    jvs[497 * s] = 0.0 - (r[86 * s] * v[150 * s]);
    jvs[498 * s] = 0.0 - (r[238 * s] * v[150 * s]);
    jvs[499 * s] = 0.0 - (r[234 * s] * v[150 * s]);
    jvs[500 * s] = 0.0 + (r[52 * s]);
    jvs[501 * s] = 0.0 + (r[91 * s]);
    jvs[502 * s] = 0.0 + 0x1.0000000000000p+1 * (r[87 * s] * v[158 * s]);
    jvs[503 * s] = 0.0;
    jvs[504 * s] = 0.0;
    jvs[505 * s] = 0.0 - (r[66 * s] * v[155 * s]) - (r[92 * s] * v[157 * s]) - (r[93 * s] * v[160 * s]) - (r[134 * s]);
    jvs[506 * s] = 0.0;
    jvs[507 * s] = 0.0 - (r[66 * s] * v[151 * s]);
    jvs[508 * s] = 0.0 + 0x1.0000000000000p+1 * (r[88 * s] * v[158 * s]);
    jvs[509 * s] = 0.0 - (r[92 * s] * v[151 * s]);
    jvs[510 * s] = 0.0 + 0x1.0000000000000p+1 * (r[87 * s] * v[144 * s]) + 0x1.0000000000000p+1 * (r[88 * s] * v[156 * s]) + 0x1.0000000000000p+1 * (r[89 * s] * v[159 * s]);
    jvs[511 * s] = 0.0 + 0x1.0000000000000p+1 * (r[89 * s] * v[158 * s]);
    jvs[512 * s] = 0.0 - (r[93 * s] * v[151 * s]);
    jvs[513 * s] = 0.0 + (r[45 * s]);
    jvs[514 * s] = 0.0 - (r[59 * s] * v[152 * s]);
    jvs[515 * s] = 0.0 + (r[202 * s] * v[160 * s]);
    jvs[516 * s] = 0.0;
    jvs[517 * s] = 0.0;
    jvs[518 * s] = 0.0 + (r[249 * s] * v[160 * s]);
    jvs[519 * s] = 0.0;
    jvs[520 * s] = 0.0;
    jvs[521 * s] = 0.0 + (r[251 * s] * v[159 * s]);
    jvs[522 * s] = 0.0 + (r[231 * s]);
    jvs[523 * s] = 0.0 - (r[253 * s] * v[152 * s]);
    jvs[524 * s] = 0.0;
    jvs[525 * s] = 0.0;
    jvs[526 * s] = 0.0 + (r[85 * s] * v[154 * s]) + (r[86 * s] * v[157 * s]) + (r[234 * s] * v[160 * s]);
    jvs[527 * s] = 0.0 + (r[93 * s] * v[160 * s]);
    jvs[528 * s] = 0.0 - (r[59 * s] * v[108 * s]) - (r[62 * s] * v[155 * s]) - (r[123 * s]) - (r[253 * s] * v[147 * s]);
    jvs[529 * s] = 0.0;
    jvs[530 * s] = 0.0 + (r[85 * s] * v[150 * s]);
    jvs[531 * s] = 0.0 - (r[62 * s] * v[152 * s]);
    jvs[532 * s] = 0.0;
    jvs[533 * s] = 0.0 + (r[86 * s] * v[150 * s]);
    jvs[534 * s] = 0.0;
    jvs[535 * s] = 0.0 + (r[251 * s] * v[143 * s]);
    jvs[536 * s] = 0.0 + (r[93 * s] * v[151 * s]) + (r[202 * s] * v[130 * s]) + (r[234 * s] * v[150 * s]) + (r[249 * s] * v[137 * s]);
    jvs[537 * s] = 0.0 + (r[36 * s]);
    jvs[538 * s] = 0.0 + (r[75 * s] * v[144 * s]) + (r[76 * s] * v[156 * s]) + (r[77 * s] * v[159 * s]) + (r[78 * s] * v[13 * s] * v[144 * s]) + (r[79 * s] * v[13 * s] * v[156 * s]) + (r[80 * s] * v[13 * s] * v[159 * s]);
    jvs[539 * s] = 0.0 + (r[72 * s] * v[144 * s]) + (r[73 * s] * v[156 * s]) + (r[74 * s] * v[159 * s]) + (r[78 * s] * v[12 * s] * v[144 * s]) + (r[79 * s] * v[12 * s] * v[156 * s]) + (r[80 * s] * v[12 * s] * v[159 * s]);
    jvs[540 * s] = 0.0 - (r[154 * s] * v[153 * s]);
    jvs[541 * s] = 0.0 - (r[156 * s] * v[153 * s]);
    jvs[542 * s] = 0.0 - (r[147 * s] * v[153 * s]) - (r[151 * s] * v[153 * s]);
}

KQ_HD KQ_NOINLINE void kqu_jac_8(const double* v, const double* f, const double* r, double* jvs, long long s)
{
    jvs[543 * s] = 0.0 + (r[81 * s] * v[155 * s] * v[156 * s]);
    jvs[544 * s] = 0.0 + (r[82 * s] * v[155 * s] * v[156 * s]) + (r[83 * s] * v[156 * s]);
    jvs[545 * s] = 0.0 + (r[50 * s]);
    jvs[546 * s] = 0.0 - (r[240 * s] * v[153 * s]);
    jvs[547 * s] = 0.0 + 0x1.0000000000000p+1 * (r[245 * s] * v[155 * s] * v[156 * s]);
    jvs[548 * s] = 0.0;
    jvs[549 * s] = 0.0 + (r[69 * s] * v[157 * s]) + (r[72 * s] * v[13 * s]) + (r[75 * s] * v[12 * s]) + (r[78 * s] * v[12 * s] * v[13 * s]) + (r[87 * s] * v[158 * s]);
    jvs[550 * s] = 0.0 + (r[68 * s] * v[155 * s] * v[156 * s]);
    jvs[551 * s] = 0.0;
    jvs[552 * s] = 0.0 + (r[90 * s] * v[156 * s]);
    jvs[553 * s] = 0.0;
    jvs[554 * s] = 0.0;
    jvs[555 * s] = 0.0 - (r[64 * s] * v[155 * s]) - (r[108 * s]) - (r[147 * s] * v[115 * s]) - (r[151 * s] * v[115 * s]) - (r[154 * s] * v[75 * s]) - (r[156 * s] * v[77 * s]) - (r[240 * s] * v[126 * s]);
    jvs[556 * s] = 0.0;
    jvs[557 * s] = 0.0 - (r[64 * s] * v[153 * s]) + (r[68 * s] * v[145 * s] * v[156 * s]) + (r[81 * s] * v[120 * s] * v[156 * s]) + (r[82 * s] * v[121 * s] * v[156 * s]) + 0x1.0000000000000p+1 * (r[245 * s] * v[127 * s] * v[156 * s]);
    jvs[558 * s] = 0.0 + (r[68 * s] * v[145 * s] * v[155 * s]) + (r[70 * s] * v[157 * s]) + (r[73 * s] * v[13 * s]) + (r[76 * s] * v[12 * s]) + (r[79 * s] * v[12 * s] * v[13 * s]) + (r[81 * s] * v[120 * s] * v[155 * s]) + (r[82 * s] * v[121 * s] * v[155 * s]) + (r[83 * s] * v[121 * s]) + (r[88 * s] * v[158 * s]) + (r[90 * s] * v[149 * s]) + 0x1.0000000000000p+1 * (r[245 * s] * v[127 * s] * v[155 * s]);
    jvs[559 * s] = 0.0 + (r[69 * s] * v[144 * s]) + (r[70 * s] * v[156 * s]) + (r[71 * s] * v[159 * s]);
    jvs[560 * s] = 0.0 + (r[87 * s] * v[144 * s]) + (r[88 * s] * v[156 * s]) + (r[89 * s] * v[159 * s]);
    jvs[561 * s] = 0.0 + (r[71 * s] * v[157 * s]) + (r[74 * s] * v[13 * s]) + (r[77 * s] * v[12 * s]) + (r[80 * s] * v[12 * s] * v[13 * s]) + (r[89 * s] * v[158 * s]);
    jvs[562 * s] = 0.0;
    jvs[563 * s] = 0.0 + (r[12 * s]);
    jvs[564 * s] = 0.0 + (r[193 * s] * v[160 * s]) + (r[194 * s] * v[160 * s]);
    jvs[565 * s] = 0.0 + (r[197 * s] * v[160 * s]);
    jvs[566 * s] = 0.0 + (r[203 * s] * v[160 * s]);
    jvs[567 * s] = 0.0 + 0x1.0000000000000p+1 * (r[247 * s] * 0x1.0000000000000p+1 * v[119 * s]);
    jvs[568 * s] = 0.0 + (r[205 * s] * v[160 * s]);
    jvs[569 * s] = 0.0 + (r[204 * s] * v[160 * s]);
    jvs[570 * s] = 0.0 + (r[198 * s] * v[160 * s]);
    jvs[571 * s] = 0.0 + (r[249 * s] * v[160 * s]);
    jvs[572 * s] = 0.0 + (r[195 * s] * v[160 * s]);
    jvs[573 * s] = 0.0 + (r[196 * s] * v[160 * s]);
    jvs[574 * s] = 0.0 + (r[199 * s] * v[160 * s]);
    jvs[575 * s] = 0.0 + (r[209 * s] * v[160 * s]);
    jvs[576 * s] = 0.0 - (r[243 * s] * v[154 * s]);
    jvs[577 * s] = 0.0 + (r[235 * s] * v[160 * s]);
    jvs[578 * s] = 0.0 + (r[254 * s] * v[160 * s]);
    jvs[579 * s] = 0.0 + (r[208 * s] * v[160 * s]);
    jvs[580 * s] = 0.0 + (r[239 * s]);
    jvs[581 * s] = 0.0 + (r[65 * s] * v[155 * s]) - (r[85 * s] * v[154 * s]);
    jvs[582 * s] = 0.0;
    jvs[583 * s] = 0.0;
}

KQ_HD KQ_NOINLINE void kqu_jac_9(const double* v, const double* f, const double* r, double* jvs, long long s)
{
    jvs[584 * s] = 0.0 - (r[28 * s]) - (r[51 * s]) + -0x1.0000000000000p+1 * (r[84 * s] * 0x1.0000000000000p+1 * v[154 * s]) - (r[85 * s] * v[150 * s]) - (r[131 * s]) - (r[233 * s] * v[160 * s]) - (r[237 * s] * v[158 * s]) - (r[243 * s] * v[142 * s]);
    jvs[585 * s] = 0.0 + (r[65 * s] * v[150 * s]);
    jvs[586 * s] = 0.0;
    jvs[587 * s] = 0.0;
    jvs[588 * s] = 0.0 - (r[237 * s] * v[154 * s]);
    jvs[589 * s] = 0.0;
    jvs[590 * s] = 0.0 + (r[193 * s] * v[104 * s]) + (r[194 * s] * v[104 * s]) + (r[195 * s] * v[138 * s]) + (r[196 * s] * v[139 * s]) + (r[197 * s] * v[105 * s]) + (r[198 * s] * v[136 * s]) + (r[199 * s] * v[140 * s]) + (r[203 * s] * v[112 * s]) + (r[204 * s] * v[133 * s]) + (r[205 * s] * v[132 * s]) + (r[208 * s] * v[148 * s]) + (r[209 * s] * v[141 * s]) - (r[233 * s] * v[154 * s]) + (r[235 * s] * v[145 * s]) + (r[249 * s] * v[137 * s]) + (r[254 * s] * v[147 * s]);
    jvs[591 * s] = 0.0 + 0x1.0000000000000p+1 * (r[75 * s] * v[144 * s]) + (r[76 * s] * v[156 * s]) + 0x1.0000000000000p+1 * (r[78 * s] * v[13 * s] * v[144 * s]) + (r[79 * s] * v[13 * s] * v[156 * s]);
    jvs[592 * s] = 0.0 + 0x1.0000000000000p+1 * (r[72 * s] * v[144 * s]) + (r[73 * s] * v[156 * s]) + 0x1.0000000000000p+1 * (r[78 * s] * v[12 * s] * v[144 * s]) + (r[79 * s] * v[12 * s] * v[156 * s]);
    jvs[593 * s] = 0.0 + (r[42 * s]);
    jvs[594 * s] = 0.0 + (r[49 * s]);
    jvs[595 * s] = 0.0 + (r[47 * s]);
    jvs[596 * s] = 0.0 - (r[61 * s] * v[155 * s]);
    jvs[597 * s] = 0.0 - (r[58 * s] * v[155 * s]);
    jvs[598 * s] = 0.0 + (r[44 * s]) - (r[57 * s] * v[155 * s]);
    jvs[599 * s] = 0.0 + (r[81 * s] * v[155 * s] * v[156 * s]);
    jvs[600 * s] = 0.0 + (r[82 * s] * v[155 * s] * v[156 * s]) + (r[83 * s] * v[156 * s]);
    jvs[601 * s] = 0.0 + (r[50 * s]) - (r[63 * s] * v[155 * s]);
    jvs[602 * s] = 0.0 + (r[43 * s]);
    jvs[603 * s] = 0.0 + (r[52 * s]);
    jvs[604 * s] = 0.0 + (r[241 * s] * v[156 * s]);
    jvs[605 * s] = 0.0 + 0x1.0000000000000p+1 * (r[245 * s] * v[155 * s] * v[156 * s]);
    jvs[606 * s] = 0.0 + (r[177 * s]);
    jvs[607 * s] = 0.0 - (r[67 * s] * v[155 * s]);
    jvs[608 * s] = 0.0 - (r[184 * s] * v[155 * s]);
    jvs[609 * s] = 0.0 + (r[178 * s]) - (r[183 * s] * v[155 * s]);
    jvs[610 * s] = 0.0 - (r[185 * s] * v[155 * s]);
    jvs[611 * s] = 0.0 + (r[179 * s]);
    jvs[612 * s] = 0.0 + (r[181 * s]);
    jvs[613 * s] = 0.0 - (r[187 * s] * v[155 * s]);
    jvs[614 * s] = 0.0 + (r[176 * s]);
    jvs[615 * s] = 0.0 - (r[60 * s] * v[155 * s]);
    jvs[616 * s] = 0.0 + (r[180 * s]) + (r[195 * s] * v[160 * s]);
    jvs[617 * s] = 0.0 - (r[186 * s] * v[155 * s]);
    jvs[618 * s] = 0.0 - (r[182 * s] * v[155 * s]);
    jvs[619 * s] = 0.0 + (r[46 * s]);
    jvs[620 * s] = 0.0;
    jvs[621 * s] = 0.0 + (r[40 * s]) + 0x1.0000000000000p+1 * (r[69 * s] * v[157 * s]) + 0x1.0000000000000p+1 * (r[72 * s] * v[13 * s]) + 0x1.0000000000000p+1 * (r[75 * s] * v[12 * s]) + 0x1.0000000000000p+1 * (r[78 * s] * v[12 * s] * v[13 * s]) + 0x1.0000000000000p+2 * (r[87 * s] * v[158 * s]);
    jvs[622 * s] = 0.0 + (r[68 * s] * v[155 * s] * v[156 * s]);
    jvs[623 * s] = 0.0 - (r[56 * s] * v[155 * s]);
    jvs[624 * s] = 0.0;
    jvs[625 * s] = 0.0;
    jvs[626 * s] = 0.0 + (r[53 * s]) + 0x1.0000000000000p+1 * (r[90 * s] * v[156 * s]);
    jvs[627 * s] = 0.0 - (r[65 * s] * v[155 * s]);
    jvs[628 * s] = 0.0 - (r[66 * s] * v[155 * s]);
    jvs[629 * s] = 0.0 - (r[62 * s] * v[155 * s]);
    jvs[630 * s] = 0.0 - (r[64 * s] * v[155 * s]);
    jvs[631 * s] = 0.0 + (r[51 * s]);
}

KQ_HD KQ_NOINLINE void kqu_jac_10(const double* v, const double* f, const double* r, double* jvs, long long s)
{
    jvs[632 * s] = 0.0 - (r[54 * s] * v[156 * s]) - (r[55 * s] * v[159 * s]) - (r[56 * s] * v[146 * s]) - (r[57 * s] * v[114 * s]) - (r[58 * s] * v[113 * s]) - (r[60 * s] * v[137 * s]) - (r[61 * s] * v[111 * s]) - (r[62 * s] * v[152 * s]) - (r[63 * s] * v[123 * s]) - (r[64 * s] * v[153 * s]) - (r[65 * s] * v[150 * s]) - (r[66 * s] * v[151 * s]) - (r[67 * s] * v[129 * s]) + (r[68 * s] * v[145 * s] * v[156 * s]) + (r[81 * s] * v[120 * s] * v[156 * s]) + (r[82 * s] * v[121 * s] * v[156 * s]) - (r[122 * s]) - (r[182 * s] * v[140 * s]) - (r[183 * s] * v[131 * s]) - (r[184 * s] * v[130 * s]) - (r[185 * s] * v[132 * s]) - (r[186 * s] * v[139 * s]) - (r[187 * s] * v[135 * s]) + 0x1.0000000000000p+1 * (r[245 * s] * v[127 * s] * v[156 * s]);
    jvs[633 * s] = 0.0 + (r[41 * s]) - (r[54 * s] * v[155 * s]) + (r[68 * s] * v[145 * s] * v[155 * s]) + (r[70 * s] * v[157 * s]) + (r[73 * s] * v[13 * s]) + (r[76 * s] * v[12 * s]) + (r[79 * s] * v[12 * s] * v[13 * s]) + (r[81 * s] * v[120 * s] * v[155 * s]) + (r[82 * s] * v[121 * s] * v[155 * s]) + (r[83 * s] * v[121 * s]) + 0x1.8000000000000p+1 * (r[88 * s] * v[158 * s]) + 0x1.0000000000000p+1 * (r[90 * s] * v[149 * s]) + (r[241 * s] * v[126 * s]) + 0x1.0000000000000p+1 * (r[245 * s] * v[127 * s] * v[155 * s]);
    jvs[634 * s] = 0.0 + 0x1.0000000000000p+1 * (r[69 * s] * v[144 * s]) + (r[70 * s] * v[156 * s]);
    jvs[635 * s] = 0.0 + 0x1.0000000000000p+2 * (r[87 * s] * v[144 * s]) + 0x1.8000000000000p+1 * (r[88 * s] * v[156 * s]) + 0x1.0000000000000p+1 * (r[89 * s] * v[159 * s]);
    jvs[636 * s] = 0.0 - (r[55 * s] * v[155 * s]) + 0x1.0000000000000p+1 * (r[89 * s] * v[158 * s]);
    jvs[637 * s] = 0.0 + (r[195 * s] * v[138 * s]);
    jvs[638 * s] = 0.0 - (r[76 * s] * v[156 * s]) - (r[79 * s] * v[13 * s] * v[156 * s]);
    jvs[639 * s] = 0.0 - (r[73 * s] * v[156 * s]) - (r[79 * s] * v[12 * s] * v[156 * s]);
    jvs[640 * s] = 0.0 - (r[248 * s] * v[156 * s]);
    jvs[641 * s] = 0.0 - (r[81 * s] * v[155 * s] * v[156 * s]);
    jvs[642 * s] = 0.0 - (r[82 * s] * v[155 * s] * v[156 * s]) - (r[83 * s] * v[156 * s]);
    jvs[643 * s] = 0.0 - (r[241 * s] * v[156 * s]);
    jvs[644 * s] = 0.0 - (r[245 * s] * v[155 * s] * v[156 * s]);
    jvs[645 * s] = 0.0;
    jvs[646 * s] = 0.0 - (r[250 * s] * v[156 * s]);
    jvs[647 * s] = 0.0 + (r[40 * s]);
    jvs[648 * s] = 0.0 - (r[68 * s] * v[155 * s] * v[156 * s]);
    jvs[649 * s] = 0.0 + (r[252 * s]) + (r[254 * s] * v[160 * s]);
    jvs[650 * s] = 0.0;
    jvs[651 * s] = 0.0 - (r[90 * s] * v[156 * s]);
    jvs[652 * s] = 0.0;
    jvs[653 * s] = 0.0;
    jvs[654 * s] = 0.0;
    jvs[655 * s] = 0.0;
    jvs[656 * s] = 0.0 - (r[54 * s] * v[156 * s]) + (r[55 * s] * v[159 * s]) - (r[68 * s] * v[145 * s] * v[156 * s]) - (r[81 * s] * v[120 * s] * v[156 * s]) - (r[82 * s] * v[121 * s] * v[156 * s]) - (r[245 * s] * v[127 * s] * v[156 * s]);
}

KQ_HD KQ_NOINLINE void kqu_jac_11(const double* v, const double* f, const double* r, double* jvs, long long s)
{
    jvs[657 * s] = 0.0 - (r[41 * s]) - (r[54 * s] * v[155 * s]) - (r[68 * s] * v[145 * s] * v[155 * s]) - (r[70 * s] * v[157 * s]) - (r[73 * s] * v[13 * s]) - (r[76 * s] * v[12 * s]) - (r[79 * s] * v[12 * s] * v[13 * s]) - (r[81 * s] * v[120 * s] * v[155 * s]) - (r[82 * s] * v[121 * s] * v[155 * s]) - (r[83 * s] * v[121 * s]) - (r[88 * s] * v[158 * s]) - (r[90 * s] * v[149 * s]) - (r[124 * s]) - (r[236 * s] * v[160 * s]) - (r[241 * s] * v[126 * s]) - (r[245 * s] * v[127 * s] * v[155 * s]) - (r[248 * s] * v[119 * s]) - (r[250 * s] * v[143 * s]);
    jvs[658 * s] = 0.0 - (r[70 * s] * v[156 * s]);
    jvs[659 * s] = 0.0 - (r[88 * s] * v[156 * s]);
    jvs[660 * s] = 0.0 + (r[55 * s] * v[155 * s]);
    jvs[661 * s] = 0.0 - (r[236 * s] * v[156 * s]) + (r[254 * s] * v[147 * s]);
    jvs[662 * s] = 0.0 + (r[5 * s]);
    jvs[663 * s] = 0.0 - (r[69 * s] * v[157 * s]);
    jvs[664 * s] = 0.0 - (r[86 * s] * v[157 * s]);
    jvs[665 * s] = 0.0 - (r[92 * s] * v[157 * s]);
    jvs[666 * s] = 0.0;
    jvs[667 * s] = 0.0;
    jvs[668 * s] = 0.0 - (r[70 * s] * v[157 * s]);
    jvs[669 * s] = 0.0 - (r[21 * s]) - (r[69 * s] * v[144 * s]) - (r[70 * s] * v[156 * s]) - (r[71 * s] * v[159 * s]) - (r[86 * s] * v[150 * s]) - (r[92 * s] * v[151 * s]) - (r[100 * s]);
    jvs[670 * s] = 0.0;
    jvs[671 * s] = 0.0 - (r[71 * s] * v[157 * s]);
    jvs[672 * s] = 0.0;
    jvs[673 * s] = 0.0 + (r[13 * s]);
    jvs[674 * s] = 0.0 + (r[94 * s] * v[160 * s]);
    jvs[675 * s] = 0.0 + -0x1.0000000000000p+1 * (r[87 * s] * v[158 * s]);
    jvs[676 * s] = 0.0 + (r[231 * s]);
    jvs[677 * s] = 0.0 + (r[239 * s]);
    jvs[678 * s] = 0.0 - (r[238 * s] * v[158 * s]);
    jvs[679 * s] = 0.0 + (r[93 * s] * v[160 * s]);
    jvs[680 * s] = 0.0;
    jvs[681 * s] = 0.0 - (r[237 * s] * v[158 * s]);
    jvs[682 * s] = 0.0;
    jvs[683 * s] = 0.0 + -0x1.0000000000000p+1 * (r[88 * s] * v[158 * s]);
    jvs[684 * s] = 0.0;
    jvs[685 * s] = 0.0 - (r[29 * s]) + -0x1.0000000000000p+1 * (r[87 * s] * v[144 * s]) + -0x1.0000000000000p+1 * (r[88 * s] * v[156 * s]) + -0x1.0000000000000p+1 * (r[89 * s] * v[159 * s]) - (r[132 * s]) - (r[237 * s] * v[154 * s]) - (r[238 * s] * v[150 * s]);
    jvs[686 * s] = 0.0 + -0x1.0000000000000p+1 * (r[89 * s] * v[158 * s]);
    jvs[687 * s] = 0.0 + (r[93 * s] * v[151 * s]) + (r[94 * s] * v[125 * s]);
    jvs[688 * s] = 0.0 - (r[77 * s] * v[159 * s]) - (r[80 * s] * v[13 * s] * v[159 * s]);
    jvs[689 * s] = 0.0 - (r[74 * s] * v[159 * s]) - (r[80 * s] * v[12 * s] * v[159 * s]);
    jvs[690 * s] = 0.0 - (r[251 * s] * v[159 * s]);
    jvs[691 * s] = 0.0 + (r[253 * s] * v[152 * s]);
    jvs[692 * s] = 0.0;
    jvs[693 * s] = 0.0 + (r[253 * s] * v[147 * s]);
    jvs[694 * s] = 0.0;
    jvs[695 * s] = 0.0;
    jvs[696 * s] = 0.0 - (r[55 * s] * v[159 * s]);
    jvs[697 * s] = 0.0 + (r[41 * s]);
    jvs[698 * s] = 0.0 - (r[71 * s] * v[159 * s]);
    jvs[699 * s] = 0.0 - (r[89 * s] * v[159 * s]);
    jvs[700 * s] = 0.0 - (r[55 * s] * v[155 * s]) - (r[71 * s] * v[157 * s]) - (r[74 * s] * v[13 * s]) - (r[77 * s] * v[12 * s]) - (r[80 * s] * v[12 * s] * v[13 * s]) - (r[89 * s] * v[158 * s]) - (r[125 * s]) - (r[251 * s] * v[143 * s]);
    jvs[701 * s] = 0.0;
    jvs[702 * s] = 0.0 - (r[193 * s] * v[160 * s]) - (r[194 * s] * v[160 * s]);
    jvs[703 * s] = 0.0 - (r[197 * s] * v[160 * s]);
    jvs[704 * s] = 0.0 - (r[203 * s] * v[160 * s]);
}

KQ_HD KQ_NOINLINE void kqu_jac_12(const double* v, const double* f, const double* r, double* jvs, long long s)
{
    jvs[705 * s] = 0.0 + (r[246 * s] * f[0 * s]);
    jvs[706 * s] = 0.0 - (r[94 * s] * v[160 * s]);
    jvs[707 * s] = 0.0;
    jvs[708 * s] = 0.0 + -0x1.0000000000000p+1 * (r[200 * s] * v[160 * s]);
    jvs[709 * s] = 0.0 - (r[202 * s] * v[160 * s]);
    jvs[710 * s] = 0.0 - (r[201 * s] * v[160 * s]);
    jvs[711 * s] = 0.0 - (r[205 * s] * v[160 * s]);
    jvs[712 * s] = 0.0 - (r[204 * s] * v[160 * s]);
    jvs[713 * s] = 0.0 - (r[206 * s] * v[160 * s]);
    jvs[714 * s] = 0.0 - (r[207 * s] * v[160 * s]);
    jvs[715 * s] = 0.0 - (r[198 * s] * v[160 * s]);
    jvs[716 * s] = 0.0 - (r[249 * s] * v[160 * s]);
    jvs[717 * s] = 0.0 - (r[195 * s] * v[160 * s]);
    jvs[718 * s] = 0.0 - (r[196 * s] * v[160 * s]);
    jvs[719 * s] = 0.0 - (r[199 * s] * v[160 * s]);
    jvs[720 * s] = 0.0 - (r[209 * s] * v[160 * s]);
    jvs[721 * s] = 0.0;
    jvs[722 * s] = 0.0 + 0x1.0000000000000p+1 * (r[192 * s]) - (r[235 * s] * v[160 * s]);
    jvs[723 * s] = 0.0 + (r[231 * s]);
    jvs[724 * s] = 0.0 - (r[254 * s] * v[160 * s]);
    jvs[725 * s] = 0.0 - (r[208 * s] * v[160 * s]);
    jvs[726 * s] = 0.0;
    jvs[727 * s] = 0.0 + (r[86 * s] * v[157 * s]) - (r[234 * s] * v[160 * s]);
    jvs[728 * s] = 0.0 - (r[93 * s] * v[160 * s]);
    jvs[729 * s] = 0.0;
    jvs[730 * s] = 0.0;
    jvs[731 * s] = 0.0 - (r[233 * s] * v[160 * s]);
    jvs[732 * s] = 0.0;
    jvs[733 * s] = 0.0 - (r[236 * s] * v[160 * s]);
    jvs[734 * s] = 0.0 + (r[86 * s] * v[150 * s]);
    jvs[735 * s] = 0.0;
    jvs[736 * s] = 0.0;
    jvs[737 * s] = 0.0 - (r[93 * s] * v[151 * s]) - (r[94 * s] * v[125 * s]) - (r[138 * s]) - (r[139 * s]) - (r[193 * s] * v[104 * s]) - (r[194 * s] * v[104 * s]) - (r[195 * s] * v[138 * s]) - (r[196 * s] * v[139 * s]) - (r[197 * s] * v[105 * s]) - (r[198 * s] * v[136 * s]) - (r[199 * s] * v[140 * s]) + -0x1.0000000000000p+1 * (r[200 * s] * v[128 * s]) - (r[201 * s] * v[131 * s]) - (r[202 * s] * v[130 * s]) - (r[203 * s] * v[112 * s]) - (r[204 * s] * v[133 * s]) - (r[205 * s] * v[132 * s]) - (r[206 * s] * v[134 * s]) - (r[207 * s] * v[135 * s]) - (r[208 * s] * v[148 * s]) - (r[209 * s] * v[141 * s]) + -0x1.0000000000000p+1 * (r[232 * s] * 0x1.0000000000000p+1 * v[160 * s]) - (r[233 * s] * v[154 * s]) - (r[234 * s] * v[150 * s]) - (r[235 * s] * v[145 * s]) - (r[236 * s] * v[156 * s]) - (r[249 * s] * v[137 * s]) - (r[254 * s] * v[147 * s]);
}

KQ_HD inline void kqu_jac(const double* v, const double* f, const double* r, double* jvs, long long s)
{
    kqu_jac_0(v, f, r, jvs, s);
    kqu_jac_1(v, f, r, jvs, s);
    kqu_jac_2(v, f, r, jvs, s);
    kqu_jac_3(v, f, r, jvs, s);
    kqu_jac_4(v, f, r, jvs, s);
    kqu_jac_5(v, f, r, jvs, s);
    kqu_jac_6(v, f, r, jvs, s);
    kqu_jac_7(v, f, r, jvs, s);
    kqu_jac_8(v, f, r, jvs, s);
    kqu_jac_9(v, f, r, jvs, s);
    kqu_jac_10(v, f, r, jvs, s);
    kqu_jac_11(v, f, r, jvs, s);
    kqu_jac_12(v, f, r, jvs, s);
}

KQ_HD KQ_NOINLINE int kqu_decomp_0(double* jvs, long long s)
{
    if (fabs(jvs[0 * s]) < DBL_MIN) return 1;
    if (fabs(jvs[1 * s]) < DBL_MIN) return 2;
    if (fabs(jvs[2 * s]) < DBL_MIN) return 3;
    if (fabs(jvs[3 * s]) < DBL_MIN) return 4;
    if (fabs(jvs[4 * s]) < DBL_MIN) return 5;
    if (fabs(jvs[5 * s]) < DBL_MIN) return 6;
    if (fabs(jvs[6 * s]) < DBL_MIN) return 7;
    if (fabs(jvs[7 * s]) < DBL_MIN) return 8;
    if (fabs(jvs[9 * s]) < DBL_MIN) return 9;
    { const double a = -jvs[8 * s] / jvs[7 * s]; jvs[8 * s] = -a;
    }
    if (fabs(jvs[11 * s]) < DBL_MIN) return 10;
    { const double a = -jvs[10 * s] / jvs[5 * s]; jvs[10 * s] = -a;
    }
    if (fabs(jvs[12 * s]) < DBL_MIN) return 11;
    if (fabs(jvs[14 * s]) < DBL_MIN) return 12;
    { const double a = -jvs[13 * s] / jvs[6 * s]; jvs[13 * s] = -a;
    }
    if (fabs(jvs[15 * s]) < DBL_MIN) return 13;
    if (fabs(jvs[16 * s]) < DBL_MIN) return 14;
    if (fabs(jvs[17 * s]) < DBL_MIN) return 15;
    if (fabs(jvs[18 * s]) < DBL_MIN) return 16;
    if (fabs(jvs[19 * s]) < DBL_MIN) return 17;
    if (fabs(jvs[21 * s]) < DBL_MIN) return 18;
    { const double a = -jvs[20 * s] / jvs[3 * s]; jvs[20 * s] = -a;
    }
    if (fabs(jvs[22 * s]) < DBL_MIN) return 19;
    if (fabs(jvs[31 * s]) < DBL_MIN) return 20;
    if (fabs(jvs[33 * s]) < DBL_MIN) return 21;
    if (fabs(jvs[38 * s]) < DBL_MIN) return 22;
    if (fabs(jvs[42 * s]) < DBL_MIN) return 23;
    if (fabs(jvs[44 * s]) < DBL_MIN) return 24;
    if (fabs(jvs[46 * s]) < DBL_MIN) return 25;
    if (fabs(jvs[48 * s]) < DBL_MIN) return 26;
    if (fabs(jvs[51 * s]) < DBL_MIN) return 27;
    if (fabs(jvs[53 * s]) < DBL_MIN) return 28;
    if (fabs(jvs[55 * s]) < DBL_MIN) return 29;
    if (fabs(jvs[59 * s]) < DBL_MIN) return 30;
    if (fabs(jvs[61 * s]) < DBL_MIN) return 31;
    if (fabs(jvs[63 * s]) < DBL_MIN) return 32;
    if (fabs(jvs[65 * s]) < DBL_MIN) return 33;
    if (fabs(jvs[67 * s]) < DBL_MIN) return 34;
    if (fabs(jvs[69 * s]) < DBL_MIN) return 35;
    if (fabs(jvs[71 * s]) < DBL_MIN) return 36;
    if (fabs(jvs[74 * s]) < DBL_MIN) return 37;
    { const double a = -jvs[73 * s] / jvs[9 * s]; jvs[73 * s] = -a;
    }
    if (fabs(jvs[76 * s]) < DBL_MIN) return 38;
    { const double a = -jvs[75 * s] / jvs[15 * s]; jvs[75 * s] = -a;
    }
    if (fabs(jvs[78 * s]) < DBL_MIN) return 39;
    { const double a = -jvs[77 * s] / jvs[16 * s]; jvs[77 * s] = -a;
    }
    if (fabs(jvs[80 * s]) < DBL_MIN) return 40;
    { const double a = -jvs[79 * s] / jvs[11 * s]; jvs[79 * s] = -a;
    }
    if (fabs(jvs[82 * s]) < DBL_MIN) return 41;
    { const double a = -jvs[81 * s] / jvs[12 * s]; jvs[81 * s] = -a;
    }
    if (fabs(jvs[84 * s]) < DBL_MIN) return 42;
    { const double a = -jvs[83 * s] / jvs[14 * s]; jvs[83 * s] = -a;
    }
    if (fabs(jvs[85 * s]) < DBL_MIN) return 43;
    if (fabs(jvs[88 * s]) < DBL_MIN) return 44;
    { const double a = -jvs[87 * s] / jvs[17 * s]; jvs[87 * s] = -a;
    }
    if (fabs(jvs[90 * s]) < DBL_MIN) return 45;
    { const double a = -jvs[89 * s] / jvs[18 * s]; jvs[89 * s] = -a;
    }
    if (fabs(jvs[92 * s]) < DBL_MIN) return 46;
    { const double a = -jvs[91 * s] / jvs[19 * s]; jvs[91 * s] = -a;
    }
    if (fabs(jvs[94 * s]) < DBL_MIN) return 47;
    { const double a = -jvs[93 * s] / jvs[21 * s]; jvs[93 * s] = -a;
    }
    if (fabs(jvs[95 * s]) < DBL_MIN) return 48;
    if (fabs(jvs[97 * s]) < DBL_MIN) return 49;
    if (fabs(jvs[100 * s]) < DBL_MIN) return 50;
    if (fabs(jvs[103 * s]) < DBL_MIN) return 51;
    if (fabs(jvs[105 * s]) < DBL_MIN) return 52;
    if (fabs(jvs[108 * s]) < DBL_MIN) return 53;
    if (fabs(jvs[112 * s]) < DBL_MIN) return 54;
    if (fabs(jvs[114 * s]) < DBL_MIN) return 55;
    if (fabs(jvs[116 * s]) < DBL_MIN) return 56;
    if (fabs(jvs[120 * s]) < DBL_MIN) return 57;
    if (fabs(jvs[122 * s]) < DBL_MIN) return 58;
    if (fabs(jvs[124 * s]) < DBL_MIN) return 59;
    if (fabs(jvs[126 * s]) < DBL_MIN) return 60;
    if (fabs(jvs[129 * s]) < DBL_MIN) return 61;
    if (fabs(jvs[131 * s]) < DBL_MIN) return 62;
    if (fabs(jvs[135 * s]) < DBL_MIN) return 63;
    if (fabs(jvs[138 * s]) < DBL_MIN) return 64;
    if (fabs(jvs[142 * s]) < DBL_MIN) return 65;
    if (fabs(jvs[145 * s]) < DBL_MIN) return 66;
    if (fabs(jvs[148 * s]) < DBL_MIN) return 67;
    if (fabs(jvs[152 * s]) < DBL_MIN) return 68;
    if (fabs(jvs[155 * s]) < DBL_MIN) return 69;
    if (fabs(jvs[157 * s]) < DBL_MIN) return 70;
    if (fabs(jvs[160 * s]) < DBL_MIN) return 71;
    if (fabs(jvs[164 * s]) < DBL_MIN) return 72;
    if (fabs(jvs[166 * s]) < DBL_MIN) return 73;
    if (fabs(jvs[168 * s]) < DBL_MIN) return 74;
    if (fabs(jvs[170 * s]) < DBL_MIN) return 75;
    if (fabs(jvs[173 * s]) < DBL_MIN) return 76;
    { const double a = -jvs[172 * s] / jvs[170 * s]; jvs[172 * s] = -a;
      jvs[173 * s] = jvs[173 * s] + a * jvs[171 * s];
    }
    if (fabs(jvs[175 * s]) < DBL_MIN) return 77;
    if (fabs(jvs[178 * s]) < DBL_MIN) return 78;
    { const double a = -jvs[177 * s] / jvs[175 * s]; jvs[177 * s] = -a;
      jvs[178 * s] = jvs[178 * s] + a * jvs[176 * s];
    }
    if (fabs(jvs[180 * s]) < DBL_MIN) return 79;
    if (fabs(jvs[182 * s]) < DBL_MIN) return 80;
    if (fabs(jvs[184 * s]) < DBL_MIN) return 81;
    if (fabs(jvs[186 * s]) < DBL_MIN) return 82;
    if (fabs(jvs[188 * s]) < DBL_MIN) return 83;
    if (fabs(jvs[190 * s]) < DBL_MIN) return 84;
    if (fabs(jvs[192 * s]) < DBL_MIN) return 85;
    if (fabs(jvs[194 * s]) < DBL_MIN) return 86;
    if (fabs(jvs[196 * s]) < DBL_MIN) return 87;
    if (fabs(jvs[198 * s]) < DBL_MIN) return 88;
    if (fabs(jvs[200 * s]) < DBL_MIN) return 89;
    if (fabs(jvs[202 * s]) < DBL_MIN) return 90;
    if (fabs(jvs[204 * s]) < DBL_MIN) return 91;
    if (fabs(jvs[206 * s]) < DBL_MIN) return 92;
    if (fabs(jvs[208 * s]) < DBL_MIN) return 93;
    if (fabs(jvs[210 * s]) < DBL_MIN) return 94;
    if (fabs(jvs[212 * s]) < DBL_MIN) return 95;
    if (fabs(jvs[214 * s]) < DBL_MIN) return 96;
    if (fabs(jvs[216 * s]) < DBL_MIN) return 97;
    if (fabs(jvs[218 * s]) < DBL_MIN) return 98;
    if (fabs(jvs[220 * s]) < DBL_MIN) return 99;
    if (fabs(jvs[222 * s]) < DBL_MIN) return 100;
    if (fabs(jvs[224 * s]) < DBL_MIN) return 101;
    if (fabs(jvs[226 * s]) < DBL_MIN) return 102;
    if (fabs(jvs[228 * s]) < DBL_MIN) return 103;
    if (fabs(jvs[231 * s]) < DBL_MIN) return 104;
    if (fabs(jvs[237 * s]) < DBL_MIN) return 105;
    { const double a = -jvs[236 * s] / jvs[180 * s]; jvs[236 * s] = -a;
      jvs[237 * s] = jvs[237 * s] + a * jvs[181 * s];
    }
    if (fabs(jvs[241 * s]) < DBL_MIN) return 106;
    { const double a = -jvs[239 * s] / jvs[210 * s]; jvs[239 * s] = -a;
      jvs[241 * s] = jvs[241 * s] + a * jvs[211 * s];
    }
    { const double a = -jvs[240 * s] / jvs[237 * s]; jvs[240 * s] = -a;
      jvs[242 * s] = jvs[242 * s] + a * jvs[238 * s];
    }
    if (fabs(jvs[244 * s]) < DBL_MIN) return 107;
    { const double a = -jvs[243 * s] / jvs[194 * s]; jvs[243 * s] = -a;
      jvs[244 * s] = jvs[244 * s] + a * jvs[195 * s];
    }
    if (fabs(jvs[248 * s]) < DBL_MIN) return 108;
    { const double a = -jvs[247 * s] / jvs[198 * s]; jvs[247 * s] = -a;
      jvs[248 * s] = jvs[248 * s] + a * jvs[199 * s];
    }
    if (fabs(jvs[253 * s]) < DBL_MIN) return 109;
    { const double a = -jvs[251 * s] / jvs[1 * s]; jvs[251 * s] = -a;
    }
    { const double a = -jvs[252 * s] / jvs[248 * s]; jvs[252 * s] = -a;
      jvs[253 * s] = jvs[253 * s] + a * jvs[249 * s];
      jvs[254 * s] = jvs[254 * s] + a * jvs[250 * s];
    }
    if (fabs(jvs[255 * s]) < DBL_MIN) return 110;
    if (fabs(jvs[259 * s]) < DBL_MIN) return 111;
    { const double a = -jvs[258 * s] / jvs[208 * s]; jvs[258 * s] = -a;
      jvs[259 * s] = jvs[259 * s] + a * jvs[209 * s];
    }
    if (fabs(jvs[264 * s]) < DBL_MIN) return 112;
    { const double a = -jvs[262 * s] / jvs[2 * s]; jvs[262 * s] = -a;
    }
    { const double a = -jvs[263 * s] / jvs[259 * s]; jvs[263 * s] = -a;
      jvs[264 * s] = jvs[264 * s] + a * jvs[260 * s];
      jvs[265 * s] = jvs[265 * s] + a * jvs[261 * s];
    }
    if (fabs(jvs[267 * s]) < DBL_MIN) return 113;
    { const double a = -jvs[266 * s] / jvs[212 * s]; jvs[266 * s] = -a;
      jvs[267 * s] = jvs[267 * s] + a * jvs[213 * s];
    }
    if (fabs(jvs[269 * s]) < DBL_MIN) return 114;
    if (fabs(jvs[273 * s]) < DBL_MIN) return 115;
    { const double a = -jvs[272 * s] / jvs[269 * s]; jvs[272 * s] = -a;
      jvs[273 * s] = jvs[273 * s] + a * jvs[270 * s];
      jvs[275 * s] = jvs[275 * s] + a * jvs[271 * s];
    }
    if (fabs(jvs[279 * s]) < DBL_MIN) return 116;
    { const double a = -jvs[276 * s] / jvs[224 * s]; jvs[276 * s] = -a;
      jvs[279 * s] = jvs[279 * s] + a * jvs[225 * s];
    }
    { const double a = -jvs[277 * s] / jvs[226 * s]; jvs[277 * s] = -a;
      jvs[279 * s] = jvs[279 * s] + a * jvs[227 * s];
    }
    { const double a = -jvs[278 * s] / jvs[228 * s]; jvs[278 * s] = -a;
      jvs[279 * s] = jvs[279 * s] + a * jvs[229 * s];
      jvs[281 * s] = jvs[281 * s] + a * jvs[230 * s];
    }
    if (fabs(jvs[282 * s]) < DBL_MIN) return 117;
    if (fabs(jvs[287 * s]) < DBL_MIN) return 118;
    if (fabs(jvs[296 * s]) < DBL_MIN) return 119;
    { const double a = -jvs[293 * s] / jvs[190 * s]; jvs[293 * s] = -a;
      jvs[296 * s] = jvs[296 * s] + a * jvs[191 * s];
    }
    { const double a = -jvs[294 * s] / jvs[282 * s]; jvs[294 * s] = -a;
      jvs[295 * s] = jvs[295 * s] + a * jvs[283 * s];
      jvs[296 * s] = jvs[296 * s] + a * jvs[284 * s];
      jvs[297 * s] = jvs[297 * s] + a * jvs[285 * s];
      jvs[300 * s] = jvs[300 * s] + a * jvs[286 * s];
    }
    { const double a = -jvs[295 * s] / jvs[287 * s]; jvs[295 * s] = -a;
      jvs[296 * s] = jvs[296 * s] + a * jvs[288 * s];
      jvs[297 * s] = jvs[297 * s] + a * jvs[289 * s];
      jvs[298 * s] = jvs[298 * s] + a * jvs[290 * s];
      jvs[299 * s] = jvs[299 * s] + a * jvs[291 * s];
      jvs[300 * s] = jvs[300 * s] + a * jvs[292 * s];
    }
    if (fabs(jvs[302 * s]) < DBL_MIN) return 120;
    { const double a = -jvs[301 * s] / jvs[220 * s]; jvs[301 * s] = -a;
      jvs[302 * s] = jvs[302 * s] + a * jvs[221 * s];
    }
    if (fabs(jvs[306 * s]) < DBL_MIN) return 121;
    { const double a = -jvs[304 * s] / jvs[204 * s]; jvs[304 * s] = -a;
      jvs[306 * s] = jvs[306 * s] + a * jvs[205 * s];
    }
    { const double a = -jvs[305 * s] / jvs[302 * s]; jvs[305 * s] = -a;
      jvs[308 * s] = jvs[308 * s] + a * jvs[303 * s];
    }
    if (fabs(jvs[310 * s]) < DBL_MIN) return 122;
    { const double a = -jvs[309 * s] / jvs[206 * s]; jvs[309 * s] = -a;
      jvs[310 * s] = jvs[310 * s] + a * jvs[207 * s];
    }
    if (fabs(jvs[313 * s]) < DBL_MIN) return 123;
    return 0;
}

KQ_HD KQ_NOINLINE int kqu_decomp_1(double* jvs, long long s)
{
    if (fabs(jvs[319 * s]) < DBL_MIN) return 124;
    { const double a = -jvs[317 * s] / jvs[255 * s]; jvs[317 * s] = -a;
      jvs[319 * s] = jvs[319 * s] + a * jvs[256 * s];
      jvs[323 * s] = jvs[323 * s] + a * jvs[257 * s];
    }
    { const double a = -jvs[318 * s] / jvs[313 * s]; jvs[318 * s] = -a;
      jvs[320 * s] = jvs[320 * s] + a * jvs[314 * s];
      jvs[321 * s] = jvs[321 * s] + a * jvs[315 * s];
      jvs[322 * s] = jvs[322 * s] + a * jvs[316 * s];
    }
    if (fabs(jvs[326 * s]) < DBL_MIN) return 125;
    { const double a = -jvs[324 * s] / jvs[196 * s]; jvs[324 * s] = -a;
      jvs[326 * s] = jvs[326 * s] + a * jvs[197 * s];
    }
    { const double a = -jvs[325 * s] / jvs[273 * s]; jvs[325 * s] = -a;
      jvs[326 * s] = jvs[326 * s] + a * jvs[274 * s];
      jvs[334 * s] = jvs[334 * s] + a * jvs[275 * s];
    }
    if (fabs(jvs[337 * s]) < DBL_MIN) return 126;
    { const double a = -jvs[336 * s] / jvs[168 * s]; jvs[336 * s] = -a;
      jvs[337 * s] = jvs[337 * s] + a * jvs[169 * s];
    }
    if (fabs(jvs[342 * s]) < DBL_MIN) return 127;
    { const double a = -jvs[341 * s] / jvs[218 * s]; jvs[341 * s] = -a;
      jvs[342 * s] = jvs[342 * s] + a * jvs[219 * s];
    }
    if (fabs(jvs[345 * s]) < DBL_MIN) return 128;
    if (fabs(jvs[350 * s]) < DBL_MIN) return 129;
    if (fabs(jvs[355 * s]) < DBL_MIN) return 130;
    if (fabs(jvs[360 * s]) < DBL_MIN) return 131;
    if (fabs(jvs[366 * s]) < DBL_MIN) return 132;
    { const double a = -jvs[364 * s] / jvs[350 * s]; jvs[364 * s] = -a;
      jvs[366 * s] = jvs[366 * s] + a * jvs[351 * s];
      jvs[367 * s] = jvs[367 * s] + a * jvs[352 * s];
      jvs[369 * s] = jvs[369 * s] + a * jvs[353 * s];
      jvs[370 * s] = jvs[370 * s] + a * jvs[354 * s];
    }
    { const double a = -jvs[365 * s] / jvs[360 * s]; jvs[365 * s] = -a;
      jvs[366 * s] = jvs[366 * s] + a * jvs[361 * s];
      jvs[369 * s] = jvs[369 * s] + a * jvs[362 * s];
      jvs[370 * s] = jvs[370 * s] + a * jvs[363 * s];
    }
    if (fabs(jvs[372 * s]) < DBL_MIN) return 133;
    { const double a = -jvs[371 * s] / jvs[267 * s]; jvs[371 * s] = -a;
      jvs[375 * s] = jvs[375 * s] + a * jvs[268 * s];
    }
    if (fabs(jvs[378 * s]) < DBL_MIN) return 134;
    { const double a = -jvs[376 * s] / jvs[188 * s]; jvs[376 * s] = -a;
      jvs[378 * s] = jvs[378 * s] + a * jvs[189 * s];
    }
    { const double a = -jvs[377 * s] / jvs[372 * s]; jvs[377 * s] = -a;
      jvs[378 * s] = jvs[378 * s] + a * jvs[373 * s];
      jvs[379 * s] = jvs[379 * s] + a * jvs[374 * s];
      jvs[380 * s] = jvs[380 * s] + a * jvs[375 * s];
    }
    if (fabs(jvs[383 * s]) < DBL_MIN) return 135;
    { const double a = -jvs[381 * s] / jvs[182 * s]; jvs[381 * s] = -a;
      jvs[383 * s] = jvs[383 * s] + a * jvs[183 * s];
    }
    { const double a = -jvs[382 * s] / jvs[378 * s]; jvs[382 * s] = -a;
      jvs[385 * s] = jvs[385 * s] + a * jvs[379 * s];
      jvs[386 * s] = jvs[386 * s] + a * jvs[380 * s];
    }
    if (fabs(jvs[390 * s]) < DBL_MIN) return 136;
    { const double a = -jvs[387 * s] / jvs[372 * s]; jvs[387 * s] = -a;
      jvs[388 * s] = jvs[388 * s] + a * jvs[373 * s];
      jvs[391 * s] = jvs[391 * s] + a * jvs[374 * s];
      jvs[392 * s] = jvs[392 * s] + a * jvs[375 * s];
    }
    { const double a = -jvs[388 * s] / jvs[378 * s]; jvs[388 * s] = -a;
      jvs[391 * s] = jvs[391 * s] + a * jvs[379 * s];
      jvs[392 * s] = jvs[392 * s] + a * jvs[380 * s];
    }
    { const double a = -jvs[389 * s] / jvs[383 * s]; jvs[389 * s] = -a;
      jvs[390 * s] = jvs[390 * s] + a * jvs[384 * s];
      jvs[391 * s] = jvs[391 * s] + a * jvs[385 * s];
      jvs[392 * s] = jvs[392 * s] + a * jvs[386 * s];
    }
    if (fabs(jvs[396 * s]) < DBL_MIN) return 137;
    { const double a = -jvs[393 * s] / jvs[241 * s]; jvs[393 * s] = -a;
      jvs[399 * s] = jvs[399 * s] + a * jvs[242 * s];
    }
    { const double a = -jvs[394 * s] / jvs[383 * s]; jvs[394 * s] = -a;
      jvs[395 * s] = jvs[395 * s] + a * jvs[384 * s];
      jvs[398 * s] = jvs[398 * s] + a * jvs[385 * s];
      jvs[399 * s] = jvs[399 * s] + a * jvs[386 * s];
    }
    { const double a = -jvs[395 * s] / jvs[390 * s]; jvs[395 * s] = -a;
      jvs[398 * s] = jvs[398 * s] + a * jvs[391 * s];
      jvs[399 * s] = jvs[399 * s] + a * jvs[392 * s];
    }
    if (fabs(jvs[400 * s]) < DBL_MIN) return 138;
    if (fabs(jvs[405 * s]) < DBL_MIN) return 139;
    { const double a = -jvs[404 * s] / jvs[237 * s]; jvs[404 * s] = -a;
      jvs[408 * s] = jvs[408 * s] + a * jvs[238 * s];
    }
    if (fabs(jvs[410 * s]) < DBL_MIN) return 140;
    { const double a = -jvs[409 * s] / jvs[405 * s]; jvs[409 * s] = -a;
      jvs[410 * s] = jvs[410 * s] + a * jvs[406 * s];
      jvs[411 * s] = jvs[411 * s] + a * jvs[407 * s];
      jvs[412 * s] = jvs[412 * s] + a * jvs[408 * s];
    }
    if (fabs(jvs[418 * s]) < DBL_MIN) return 141;
    { const double a = -jvs[413 * s] / jvs[267 * s]; jvs[413 * s] = -a;
      jvs[420 * s] = jvs[420 * s] + a * jvs[268 * s];
    }
    { const double a = -jvs[414 * s] / jvs[390 * s]; jvs[414 * s] = -a;
      jvs[419 * s] = jvs[419 * s] + a * jvs[391 * s];
      jvs[420 * s] = jvs[420 * s] + a * jvs[392 * s];
    }
    { const double a = -jvs[415 * s] / jvs[396 * s]; jvs[415 * s] = -a;
      jvs[418 * s] = jvs[418 * s] + a * jvs[397 * s];
      jvs[419 * s] = jvs[419 * s] + a * jvs[398 * s];
      jvs[420 * s] = jvs[420 * s] + a * jvs[399 * s];
    }
    { const double a = -jvs[416 * s] / jvs[405 * s]; jvs[416 * s] = -a;
      jvs[417 * s] = jvs[417 * s] + a * jvs[406 * s];
      jvs[419 * s] = jvs[419 * s] + a * jvs[407 * s];
      jvs[420 * s] = jvs[420 * s] + a * jvs[408 * s];
    }
    { const double a = -jvs[417 * s] / jvs[410 * s]; jvs[417 * s] = -a;
      jvs[419 * s] = jvs[419 * s] + a * jvs[411 * s];
      jvs[420 * s] = jvs[420 * s] + a * jvs[412 * s];
    }
    if (fabs(jvs[423 * s]) < DBL_MIN) return 142;
    { const double a = -jvs[421 * s] / jvs[202 * s]; jvs[421 * s] = -a;
      jvs[423 * s] = jvs[423 * s] + a * jvs[203 * s];
    }
    { const double a = -jvs[422 * s] / jvs[400 * s]; jvs[422 * s] = -a;
      jvs[423 * s] = jvs[423 * s] + a * jvs[401 * s];
      jvs[426 * s] = jvs[426 * s] + a * jvs[402 * s];
      jvs[427 * s] = jvs[427 * s] + a * jvs[403 * s];
    }
    if (fabs(jvs[431 * s]) < DBL_MIN) return 143;
    { const double a = -jvs[428 * s] / jvs[231 * s]; jvs[428 * s] = -a;
      jvs[429 * s] = jvs[429 * s] + a * jvs[232 * s];
      jvs[430 * s] = jvs[430 * s] + a * jvs[233 * s];
      jvs[434 * s] = jvs[434 * s] + a * jvs[234 * s];
      jvs[435 * s] = jvs[435 * s] + a * jvs[235 * s];
    }
    { const double a = -jvs[429 * s] / jvs[302 * s]; jvs[429 * s] = -a;
      jvs[434 * s] = jvs[434 * s] + a * jvs[303 * s];
    }
    { const double a = -jvs[430 * s] / jvs[342 * s]; jvs[430 * s] = -a;
      jvs[432 * s] = jvs[432 * s] + a * jvs[343 * s];
      jvs[434 * s] = jvs[434 * s] + a * jvs[344 * s];
    }
    if (fabs(jvs[438 * s]) < DBL_MIN) return 144;
    { const double a = -jvs[436 * s] / jvs[184 * s]; jvs[436 * s] = -a;
      jvs[438 * s] = jvs[438 * s] + a * jvs[185 * s];
    }
    { const double a = -jvs[437 * s] / jvs[302 * s]; jvs[437 * s] = -a;
      jvs[441 * s] = jvs[441 * s] + a * jvs[303 * s];
    }
    if (fabs(jvs[446 * s]) < DBL_MIN) return 145;
    { const double a = -jvs[443 * s] / jvs[15 * s]; jvs[443 * s] = -a;
    }
    { const double a = -jvs[444 * s] / jvs[16 * s]; jvs[444 * s] = -a;
    }
    { const double a = -jvs[445 * s] / jvs[222 * s]; jvs[445 * s] = -a;
      jvs[446 * s] = jvs[446 * s] + a * jvs[223 * s];
    }
    if (fabs(jvs[452 * s]) < DBL_MIN) return 146;
    { const double a = -jvs[451 * s] / jvs[192 * s]; jvs[451 * s] = -a;
      jvs[452 * s] = jvs[452 * s] + a * jvs[193 * s];
    }
    if (fabs(jvs[462 * s]) < DBL_MIN) return 147;
    { const double a = -jvs[458 * s] / jvs[0 * s]; jvs[458 * s] = -a;
    }
    { const double a = -jvs[459 * s] / jvs[244 * s]; jvs[459 * s] = -a;
      jvs[462 * s] = jvs[462 * s] + a * jvs[245 * s];
      jvs[466 * s] = jvs[466 * s] + a * jvs[246 * s];
    }
    { const double a = -jvs[460 * s] / jvs[279 * s]; jvs[460 * s] = -a;
      jvs[462 * s] = jvs[462 * s] + a * jvs[280 * s];
      jvs[465 * s] = jvs[465 * s] + a * jvs[281 * s];
    }
    { const double a = -jvs[461 * s] / jvs[342 * s]; jvs[461 * s] = -a;
      jvs[465 * s] = jvs[465 * s] + a * jvs[343 * s];
      jvs[467 * s] = jvs[467 * s] + a * jvs[344 * s];
    }
    if (fabs(jvs[470 * s]) < DBL_MIN) return 148;
    { const double a = -jvs[469 * s] / jvs[438 * s]; jvs[469 * s] = -a;
      jvs[470 * s] = jvs[470 * s] + a * jvs[439 * s];
      jvs[471 * s] = jvs[471 * s] + a * jvs[440 * s];
      jvs[473 * s] = jvs[473 * s] + a * jvs[441 * s];
      jvs[474 * s] = jvs[474 * s] + a * jvs[442 * s];
    }
    if (fabs(jvs[480 * s]) < DBL_MIN) return 149;
    { const double a = -jvs[476 * s] / jvs[383 * s]; jvs[476 * s] = -a;
      jvs[477 * s] = jvs[477 * s] + a * jvs[384 * s];
      jvs[482 * s] = jvs[482 * s] + a * jvs[385 * s];
      jvs[485 * s] = jvs[485 * s] + a * jvs[386 * s];
    }
    { const double a = -jvs[477 * s] / jvs[390 * s]; jvs[477 * s] = -a;
      jvs[482 * s] = jvs[482 * s] + a * jvs[391 * s];
      jvs[485 * s] = jvs[485 * s] + a * jvs[392 * s];
    }
    { const double a = -jvs[478 * s] / jvs[438 * s]; jvs[478 * s] = -a;
      jvs[479 * s] = jvs[479 * s] + a * jvs[439 * s];
      jvs[480 * s] = jvs[480 * s] + a * jvs[440 * s];
      jvs[483 * s] = jvs[483 * s] + a * jvs[441 * s];
      jvs[484 * s] = jvs[484 * s] + a * jvs[442 * s];
    }
    { const double a = -jvs[479 * s] / jvs[470 * s]; jvs[479 * s] = -a;
      jvs[480 * s] = jvs[480 * s] + a * jvs[471 * s];
      jvs[481 * s] = jvs[481 * s] + a * jvs[472 * s];
      jvs[483 * s] = jvs[483 * s] + a * jvs[473 * s];
      jvs[484 * s] = jvs[484 * s] + a * jvs[474 * s];
      jvs[485 * s] = jvs[485 * s] + a * jvs[475 * s];
    }
    if (fabs(jvs[488 * s]) < DBL_MIN) return 150;
    { const double a = -jvs[486 * s] / jvs[216 * s]; jvs[486 * s] = -a;
      jvs[488 * s] = jvs[488 * s] + a * jvs[217 * s];
    }
    { const double a = -jvs[487 * s] / jvs[355 * s]; jvs[487 * s] = -a;
      jvs[488 * s] = jvs[488 * s] + a * jvs[356 * s];
      jvs[489 * s] = jvs[489 * s] + a * jvs[357 * s];
      jvs[491 * s] = jvs[491 * s] + a * jvs[358 * s];
      jvs[493 * s] = jvs[493 * s] + a * jvs[359 * s];
    }
    if (fabs(jvs[494 * s]) < DBL_MIN) return 151;
    return 0;
}

KQ_HD KQ_NOINLINE int kqu_decomp_2(double* jvs, long long s)
{
    if (fabs(jvs[505 * s]) < DBL_MIN) return 152;
    { const double a = -jvs[500 * s] / jvs[337 * s]; jvs[500 * s] = -a;
      jvs[505 * s] = jvs[505 * s] + a * jvs[338 * s];
      jvs[507 * s] = jvs[507 * s] + a * jvs[339 * s];
      jvs[512 * s] = jvs[512 * s] + a * jvs[340 * s];
    }
    { const double a = -jvs[501 * s] / jvs[355 * s]; jvs[501 * s] = -a;
      jvs[503 * s] = jvs[503 * s] + a * jvs[356 * s];
      jvs[504 * s] = jvs[504 * s] + a * jvs[357 * s];
      jvs[507 * s] = jvs[507 * s] + a * jvs[358 * s];
      jvs[510 * s] = jvs[510 * s] + a * jvs[359 * s];
    }
    { const double a = -jvs[502 * s] / jvs[446 * s]; jvs[502 * s] = -a;
      jvs[507 * s] = jvs[507 * s] + a * jvs[447 * s];
      jvs[508 * s] = jvs[508 * s] + a * jvs[448 * s];
      jvs[509 * s] = jvs[509 * s] + a * jvs[449 * s];
      jvs[510 * s] = jvs[510 * s] + a * jvs[450 * s];
    }
    { const double a = -jvs[503 * s] / jvs[488 * s]; jvs[503 * s] = -a;
      jvs[504 * s] = jvs[504 * s] + a * jvs[489 * s];
      jvs[506 * s] = jvs[506 * s] + a * jvs[490 * s];
      jvs[507 * s] = jvs[507 * s] + a * jvs[491 * s];
      jvs[508 * s] = jvs[508 * s] + a * jvs[492 * s];
      jvs[510 * s] = jvs[510 * s] + a * jvs[493 * s];
    }
    { const double a = -jvs[504 * s] / jvs[494 * s]; jvs[504 * s] = -a;
      jvs[506 * s] = jvs[506 * s] + a * jvs[495 * s];
      jvs[507 * s] = jvs[507 * s] + a * jvs[496 * s];
      jvs[509 * s] = jvs[509 * s] + a * jvs[497 * s];
      jvs[510 * s] = jvs[510 * s] + a * jvs[498 * s];
      jvs[512 * s] = jvs[512 * s] + a * jvs[499 * s];
    }
    if (fabs(jvs[528 * s]) < DBL_MIN) return 153;
    { const double a = -jvs[513 * s] / jvs[248 * s]; jvs[513 * s] = -a;
      jvs[514 * s] = jvs[514 * s] + a * jvs[249 * s];
      jvs[528 * s] = jvs[528 * s] + a * jvs[250 * s];
    }
    { const double a = -jvs[514 * s] / jvs[253 * s]; jvs[514 * s] = -a;
      jvs[528 * s] = jvs[528 * s] + a * jvs[254 * s];
    }
    { const double a = -jvs[515 * s] / jvs[360 * s]; jvs[515 * s] = -a;
      jvs[516 * s] = jvs[516 * s] + a * jvs[361 * s];
      jvs[531 * s] = jvs[531 * s] + a * jvs[362 * s];
      jvs[536 * s] = jvs[536 * s] + a * jvs[363 * s];
    }
    { const double a = -jvs[516 * s] / jvs[366 * s]; jvs[516 * s] = -a;
      jvs[517 * s] = jvs[517 * s] + a * jvs[367 * s];
      jvs[519 * s] = jvs[519 * s] + a * jvs[368 * s];
      jvs[531 * s] = jvs[531 * s] + a * jvs[369 * s];
      jvs[536 * s] = jvs[536 * s] + a * jvs[370 * s];
    }
    { const double a = -jvs[517 * s] / jvs[396 * s]; jvs[517 * s] = -a;
      jvs[519 * s] = jvs[519 * s] + a * jvs[397 * s];
      jvs[531 * s] = jvs[531 * s] + a * jvs[398 * s];
      jvs[536 * s] = jvs[536 * s] + a * jvs[399 * s];
    }
    { const double a = -jvs[518 * s] / jvs[400 * s]; jvs[518 * s] = -a;
      jvs[520 * s] = jvs[520 * s] + a * jvs[401 * s];
      jvs[531 * s] = jvs[531 * s] + a * jvs[402 * s];
      jvs[536 * s] = jvs[536 * s] + a * jvs[403 * s];
    }
    { const double a = -jvs[519 * s] / jvs[418 * s]; jvs[519 * s] = -a;
      jvs[531 * s] = jvs[531 * s] + a * jvs[419 * s];
      jvs[536 * s] = jvs[536 * s] + a * jvs[420 * s];
    }
    { const double a = -jvs[520 * s] / jvs[423 * s]; jvs[520 * s] = -a;
      jvs[523 * s] = jvs[523 * s] + a * jvs[424 * s];
      jvs[524 * s] = jvs[524 * s] + a * jvs[425 * s];
      jvs[531 * s] = jvs[531 * s] + a * jvs[426 * s];
      jvs[536 * s] = jvs[536 * s] + a * jvs[427 * s];
    }
    { const double a = -jvs[521 * s] / jvs[438 * s]; jvs[521 * s] = -a;
      jvs[523 * s] = jvs[523 * s] + a * jvs[439 * s];
      jvs[524 * s] = jvs[524 * s] + a * jvs[440 * s];
      jvs[532 * s] = jvs[532 * s] + a * jvs[441 * s];
      jvs[535 * s] = jvs[535 * s] + a * jvs[442 * s];
    }
    { const double a = -jvs[522 * s] / jvs[462 * s]; jvs[522 * s] = -a;
      jvs[525 * s] = jvs[525 * s] + a * jvs[463 * s];
      jvs[527 * s] = jvs[527 * s] + a * jvs[464 * s];
      jvs[529 * s] = jvs[529 * s] + a * jvs[465 * s];
      jvs[531 * s] = jvs[531 * s] + a * jvs[466 * s];
      jvs[532 * s] = jvs[532 * s] + a * jvs[467 * s];
      jvs[533 * s] = jvs[533 * s] + a * jvs[468 * s];
    }
    { const double a = -jvs[523 * s] / jvs[470 * s]; jvs[523 * s] = -a;
      jvs[524 * s] = jvs[524 * s] + a * jvs[471 * s];
      jvs[528 * s] = jvs[528 * s] + a * jvs[472 * s];
      jvs[532 * s] = jvs[532 * s] + a * jvs[473 * s];
      jvs[535 * s] = jvs[535 * s] + a * jvs[474 * s];
      jvs[536 * s] = jvs[536 * s] + a * jvs[475 * s];
    }
    { const double a = -jvs[524 * s] / jvs[480 * s]; jvs[524 * s] = -a;
      jvs[528 * s] = jvs[528 * s] + a * jvs[481 * s];
      jvs[531 * s] = jvs[531 * s] + a * jvs[482 * s];
      jvs[532 * s] = jvs[532 * s] + a * jvs[483 * s];
      jvs[535 * s] = jvs[535 * s] + a * jvs[484 * s];
      jvs[536 * s] = jvs[536 * s] + a * jvs[485 * s];
    }
    { const double a = -jvs[525 * s] / jvs[488 * s]; jvs[525 * s] = -a;
      jvs[526 * s] = jvs[526 * s] + a * jvs[489 * s];
      jvs[530 * s] = jvs[530 * s] + a * jvs[490 * s];
      jvs[531 * s] = jvs[531 * s] + a * jvs[491 * s];
      jvs[532 * s] = jvs[532 * s] + a * jvs[492 * s];
      jvs[534 * s] = jvs[534 * s] + a * jvs[493 * s];
    }
    { const double a = -jvs[526 * s] / jvs[494 * s]; jvs[526 * s] = -a;
      jvs[530 * s] = jvs[530 * s] + a * jvs[495 * s];
      jvs[531 * s] = jvs[531 * s] + a * jvs[496 * s];
      jvs[533 * s] = jvs[533 * s] + a * jvs[497 * s];
      jvs[534 * s] = jvs[534 * s] + a * jvs[498 * s];
      jvs[536 * s] = jvs[536 * s] + a * jvs[499 * s];
    }
    { const double a = -jvs[527 * s] / jvs[505 * s]; jvs[527 * s] = -a;
      jvs[530 * s] = jvs[530 * s] + a * jvs[506 * s];
      jvs[531 * s] = jvs[531 * s] + a * jvs[507 * s];
      jvs[532 * s] = jvs[532 * s] + a * jvs[508 * s];
      jvs[533 * s] = jvs[533 * s] + a * jvs[509 * s];
      jvs[534 * s] = jvs[534 * s] + a * jvs[510 * s];
      jvs[535 * s] = jvs[535 * s] + a * jvs[511 * s];
      jvs[536 * s] = jvs[536 * s] + a * jvs[512 * s];
    }
    if (fabs(jvs[555 * s]) < DBL_MIN) return 154;
    { const double a = -jvs[537 * s] / jvs[4 * s]; jvs[537 * s] = -a;
    }
    { const double a = -jvs[538 * s] / jvs[15 * s]; jvs[538 * s] = -a;
    }
    { const double a = -jvs[539 * s] / jvs[16 * s]; jvs[539 * s] = -a;
    }
    { const double a = -jvs[540 * s] / jvs[173 * s]; jvs[540 * s] = -a;
      jvs[555 * s] = jvs[555 * s] + a * jvs[174 * s];
    }
    { const double a = -jvs[541 * s] / jvs[178 * s]; jvs[541 * s] = -a;
      jvs[555 * s] = jvs[555 * s] + a * jvs[179 * s];
    }
    { const double a = -jvs[542 * s] / jvs[279 * s]; jvs[542 * s] = -a;
      jvs[551 * s] = jvs[551 * s] + a * jvs[280 * s];
      jvs[555 * s] = jvs[555 * s] + a * jvs[281 * s];
    }
    { const double a = -jvs[543 * s] / jvs[306 * s]; jvs[543 * s] = -a;
      jvs[557 * s] = jvs[557 * s] + a * jvs[307 * s];
      jvs[558 * s] = jvs[558 * s] + a * jvs[308 * s];
    }
    { const double a = -jvs[544 * s] / jvs[310 * s]; jvs[544 * s] = -a;
      jvs[557 * s] = jvs[557 * s] + a * jvs[311 * s];
      jvs[558 * s] = jvs[558 * s] + a * jvs[312 * s];
    }
    { const double a = -jvs[545 * s] / jvs[319 * s]; jvs[545 * s] = -a;
      jvs[546 * s] = jvs[546 * s] + a * jvs[320 * s];
      jvs[548 * s] = jvs[548 * s] + a * jvs[321 * s];
      jvs[555 * s] = jvs[555 * s] + a * jvs[322 * s];
      jvs[557 * s] = jvs[557 * s] + a * jvs[323 * s];
    }
    { const double a = -jvs[546 * s] / jvs[342 * s]; jvs[546 * s] = -a;
      jvs[555 * s] = jvs[555 * s] + a * jvs[343 * s];
      jvs[558 * s] = jvs[558 * s] + a * jvs[344 * s];
    }
    { const double a = -jvs[547 * s] / jvs[345 * s]; jvs[547 * s] = -a;
      jvs[548 * s] = jvs[548 * s] + a * jvs[346 * s];
      jvs[556 * s] = jvs[556 * s] + a * jvs[347 * s];
      jvs[557 * s] = jvs[557 * s] + a * jvs[348 * s];
      jvs[558 * s] = jvs[558 * s] + a * jvs[349 * s];
    }
    { const double a = -jvs[548 * s] / jvs[431 * s]; jvs[548 * s] = -a;
      jvs[555 * s] = jvs[555 * s] + a * jvs[432 * s];
      jvs[556 * s] = jvs[556 * s] + a * jvs[433 * s];
      jvs[558 * s] = jvs[558 * s] + a * jvs[434 * s];
      jvs[562 * s] = jvs[562 * s] + a * jvs[435 * s];
    }
    { const double a = -jvs[549 * s] / jvs[446 * s]; jvs[549 * s] = -a;
      jvs[557 * s] = jvs[557 * s] + a * jvs[447 * s];
      jvs[558 * s] = jvs[558 * s] + a * jvs[448 * s];
      jvs[559 * s] = jvs[559 * s] + a * jvs[449 * s];
      jvs[560 * s] = jvs[560 * s] + a * jvs[450 * s];
    }
    { const double a = -jvs[550 * s] / jvs[452 * s]; jvs[550 * s] = -a;
      jvs[553 * s] = jvs[553 * s] + a * jvs[453 * s];
      jvs[556 * s] = jvs[556 * s] + a * jvs[454 * s];
      jvs[557 * s] = jvs[557 * s] + a * jvs[455 * s];
      jvs[558 * s] = jvs[558 * s] + a * jvs[456 * s];
      jvs[562 * s] = jvs[562 * s] + a * jvs[457 * s];
    }
    { const double a = -jvs[551 * s] / jvs[462 * s]; jvs[551 * s] = -a;
      jvs[552 * s] = jvs[552 * s] + a * jvs[463 * s];
      jvs[554 * s] = jvs[554 * s] + a * jvs[464 * s];
      jvs[555 * s] = jvs[555 * s] + a * jvs[465 * s];
      jvs[557 * s] = jvs[557 * s] + a * jvs[466 * s];
      jvs[558 * s] = jvs[558 * s] + a * jvs[467 * s];
      jvs[559 * s] = jvs[559 * s] + a * jvs[468 * s];
    }
    { const double a = -jvs[552 * s] / jvs[488 * s]; jvs[552 * s] = -a;
      jvs[553 * s] = jvs[553 * s] + a * jvs[489 * s];
      jvs[556 * s] = jvs[556 * s] + a * jvs[490 * s];
      jvs[557 * s] = jvs[557 * s] + a * jvs[491 * s];
      jvs[558 * s] = jvs[558 * s] + a * jvs[492 * s];
      jvs[560 * s] = jvs[560 * s] + a * jvs[493 * s];
    }
    { const double a = -jvs[553 * s] / jvs[494 * s]; jvs[553 * s] = -a;
      jvs[556 * s] = jvs[556 * s] + a * jvs[495 * s];
      jvs[557 * s] = jvs[557 * s] + a * jvs[496 * s];
      jvs[559 * s] = jvs[559 * s] + a * jvs[497 * s];
      jvs[560 * s] = jvs[560 * s] + a * jvs[498 * s];
      jvs[562 * s] = jvs[562 * s] + a * jvs[499 * s];
    }
    { const double a = -jvs[554 * s] / jvs[505 * s]; jvs[554 * s] = -a;
      jvs[556 * s] = jvs[556 * s] + a * jvs[506 * s];
      jvs[557 * s] = jvs[557 * s] + a * jvs[507 * s];
      jvs[558 * s] = jvs[558 * s] + a * jvs[508 * s];
      jvs[559 * s] = jvs[559 * s] + a * jvs[509 * s];
      jvs[560 * s] = jvs[560 * s] + a * jvs[510 * s];
      jvs[561 * s] = jvs[561 * s] + a * jvs[511 * s];
      jvs[562 * s] = jvs[562 * s] + a * jvs[512 * s];
    }
    return 0;
}

KQ_HD KQ_NOINLINE int kqu_decomp_3(double* jvs, long long s)
{
    if (fabs(jvs[584 * s]) < DBL_MIN) return 155;
    { const double a = -jvs[563 * s] / jvs[186 * s]; jvs[563 * s] = -a;
      jvs[584 * s] = jvs[584 * s] + a * jvs[187 * s];
    }
    { const double a = -jvs[564 * s] / jvs[237 * s]; jvs[564 * s] = -a;
      jvs[590 * s] = jvs[590 * s] + a * jvs[238 * s];
    }
    { const double a = -jvs[565 * s] / jvs[241 * s]; jvs[565 * s] = -a;
      jvs[590 * s] = jvs[590 * s] + a * jvs[242 * s];
    }
    { const double a = -jvs[566 * s] / jvs[267 * s]; jvs[566 * s] = -a;
      jvs[590 * s] = jvs[590 * s] + a * jvs[268 * s];
    }
    { const double a = -jvs[567 * s] / jvs[302 * s]; jvs[567 * s] = -a;
      jvs[586 * s] = jvs[586 * s] + a * jvs[303 * s];
    }
    { const double a = -jvs[568 * s] / jvs[372 * s]; jvs[568 * s] = -a;
      jvs[569 * s] = jvs[569 * s] + a * jvs[373 * s];
      jvs[585 * s] = jvs[585 * s] + a * jvs[374 * s];
      jvs[590 * s] = jvs[590 * s] + a * jvs[375 * s];
    }
    { const double a = -jvs[569 * s] / jvs[378 * s]; jvs[569 * s] = -a;
      jvs[585 * s] = jvs[585 * s] + a * jvs[379 * s];
      jvs[590 * s] = jvs[590 * s] + a * jvs[380 * s];
    }
    { const double a = -jvs[570 * s] / jvs[396 * s]; jvs[570 * s] = -a;
      jvs[574 * s] = jvs[574 * s] + a * jvs[397 * s];
      jvs[585 * s] = jvs[585 * s] + a * jvs[398 * s];
      jvs[590 * s] = jvs[590 * s] + a * jvs[399 * s];
    }
    { const double a = -jvs[571 * s] / jvs[400 * s]; jvs[571 * s] = -a;
      jvs[575 * s] = jvs[575 * s] + a * jvs[401 * s];
      jvs[585 * s] = jvs[585 * s] + a * jvs[402 * s];
      jvs[590 * s] = jvs[590 * s] + a * jvs[403 * s];
    }
    { const double a = -jvs[572 * s] / jvs[405 * s]; jvs[572 * s] = -a;
      jvs[573 * s] = jvs[573 * s] + a * jvs[406 * s];
      jvs[585 * s] = jvs[585 * s] + a * jvs[407 * s];
      jvs[590 * s] = jvs[590 * s] + a * jvs[408 * s];
    }
    { const double a = -jvs[573 * s] / jvs[410 * s]; jvs[573 * s] = -a;
      jvs[585 * s] = jvs[585 * s] + a * jvs[411 * s];
      jvs[590 * s] = jvs[590 * s] + a * jvs[412 * s];
    }
    { const double a = -jvs[574 * s] / jvs[418 * s]; jvs[574 * s] = -a;
      jvs[585 * s] = jvs[585 * s] + a * jvs[419 * s];
      jvs[590 * s] = jvs[590 * s] + a * jvs[420 * s];
    }
    { const double a = -jvs[575 * s] / jvs[423 * s]; jvs[575 * s] = -a;
      jvs[578 * s] = jvs[578 * s] + a * jvs[424 * s];
      jvs[579 * s] = jvs[579 * s] + a * jvs[425 * s];
      jvs[585 * s] = jvs[585 * s] + a * jvs[426 * s];
      jvs[590 * s] = jvs[590 * s] + a * jvs[427 * s];
    }
    { const double a = -jvs[576 * s] / jvs[431 * s]; jvs[576 * s] = -a;
      jvs[583 * s] = jvs[583 * s] + a * jvs[432 * s];
      jvs[584 * s] = jvs[584 * s] + a * jvs[433 * s];
      jvs[586 * s] = jvs[586 * s] + a * jvs[434 * s];
      jvs[590 * s] = jvs[590 * s] + a * jvs[435 * s];
    }
    { const double a = -jvs[577 * s] / jvs[452 * s]; jvs[577 * s] = -a;
      jvs[581 * s] = jvs[581 * s] + a * jvs[453 * s];
      jvs[584 * s] = jvs[584 * s] + a * jvs[454 * s];
      jvs[585 * s] = jvs[585 * s] + a * jvs[455 * s];
      jvs[586 * s] = jvs[586 * s] + a * jvs[456 * s];
      jvs[590 * s] = jvs[590 * s] + a * jvs[457 * s];
    }
    { const double a = -jvs[578 * s] / jvs[470 * s]; jvs[578 * s] = -a;
      jvs[579 * s] = jvs[579 * s] + a * jvs[471 * s];
      jvs[582 * s] = jvs[582 * s] + a * jvs[472 * s];
      jvs[586 * s] = jvs[586 * s] + a * jvs[473 * s];
      jvs[589 * s] = jvs[589 * s] + a * jvs[474 * s];
      jvs[590 * s] = jvs[590 * s] + a * jvs[475 * s];
    }
    { const double a = -jvs[579 * s] / jvs[480 * s]; jvs[579 * s] = -a;
      jvs[582 * s] = jvs[582 * s] + a * jvs[481 * s];
      jvs[585 * s] = jvs[585 * s] + a * jvs[482 * s];
      jvs[586 * s] = jvs[586 * s] + a * jvs[483 * s];
      jvs[589 * s] = jvs[589 * s] + a * jvs[484 * s];
      jvs[590 * s] = jvs[590 * s] + a * jvs[485 * s];
    }
    { const double a = -jvs[580 * s] / jvs[488 * s]; jvs[580 * s] = -a;
      jvs[581 * s] = jvs[581 * s] + a * jvs[489 * s];
      jvs[584 * s] = jvs[584 * s] + a * jvs[490 * s];
      jvs[585 * s] = jvs[585 * s] + a * jvs[491 * s];
      jvs[586 * s] = jvs[586 * s] + a * jvs[492 * s];
      jvs[588 * s] = jvs[588 * s] + a * jvs[493 * s];
    }
    { const double a = -jvs[581 * s] / jvs[494 * s]; jvs[581 * s] = -a;
      jvs[584 * s] = jvs[584 * s] + a * jvs[495 * s];
      jvs[585 * s] = jvs[585 * s] + a * jvs[496 * s];
      jvs[587 * s] = jvs[587 * s] + a * jvs[497 * s];
      jvs[588 * s] = jvs[588 * s] + a * jvs[498 * s];
      jvs[590 * s] = jvs[590 * s] + a * jvs[499 * s];
    }
    { const double a = -jvs[582 * s] / jvs[528 * s]; jvs[582 * s] = -a;
      jvs[583 * s] = jvs[583 * s] + a * jvs[529 * s];
      jvs[584 * s] = jvs[584 * s] + a * jvs[530 * s];
      jvs[585 * s] = jvs[585 * s] + a * jvs[531 * s];
      jvs[586 * s] = jvs[586 * s] + a * jvs[532 * s];
      jvs[587 * s] = jvs[587 * s] + a * jvs[533 * s];
      jvs[588 * s] = jvs[588 * s] + a * jvs[534 * s];
      jvs[589 * s] = jvs[589 * s] + a * jvs[535 * s];
      jvs[590 * s] = jvs[590 * s] + a * jvs[536 * s];
    }
    { const double a = -jvs[583 * s] / jvs[555 * s]; jvs[583 * s] = -a;
      jvs[584 * s] = jvs[584 * s] + a * jvs[556 * s];
      jvs[585 * s] = jvs[585 * s] + a * jvs[557 * s];
      jvs[586 * s] = jvs[586 * s] + a * jvs[558 * s];
      jvs[587 * s] = jvs[587 * s] + a * jvs[559 * s];
      jvs[588 * s] = jvs[588 * s] + a * jvs[560 * s];
      jvs[589 * s] = jvs[589 * s] + a * jvs[561 * s];
      jvs[590 * s] = jvs[590 * s] + a * jvs[562 * s];
    }
    return 0;
}

KQ_HD KQ_NOINLINE int kqu_decomp_4(double* jvs, long long s)
{
    if (fabs(jvs[632 * s]) < DBL_MIN) return 156;
    { const double a = -jvs[591 * s] / jvs[15 * s]; jvs[591 * s] = -a;
    }
    { const double a = -jvs[592 * s] / jvs[16 * s]; jvs[592 * s] = -a;
    }
    { const double a = -jvs[593 * s] / jvs[244 * s]; jvs[593 * s] = -a;
      jvs[623 * s] = jvs[623 * s] + a * jvs[245 * s];
      jvs[632 * s] = jvs[632 * s] + a * jvs[246 * s];
    }
    { const double a = -jvs[594 * s] / jvs[255 * s]; jvs[594 * s] = -a;
      jvs[601 * s] = jvs[601 * s] + a * jvs[256 * s];
      jvs[632 * s] = jvs[632 * s] + a * jvs[257 * s];
    }
    { const double a = -jvs[595 * s] / jvs[259 * s]; jvs[595 * s] = -a;
      jvs[596 * s] = jvs[596 * s] + a * jvs[260 * s];
      jvs[632 * s] = jvs[632 * s] + a * jvs[261 * s];
    }
    { const double a = -jvs[596 * s] / jvs[264 * s]; jvs[596 * s] = -a;
      jvs[632 * s] = jvs[632 * s] + a * jvs[265 * s];
    }
    { const double a = -jvs[597 * s] / jvs[269 * s]; jvs[597 * s] = -a;
      jvs[598 * s] = jvs[598 * s] + a * jvs[270 * s];
      jvs[632 * s] = jvs[632 * s] + a * jvs[271 * s];
    }
    { const double a = -jvs[598 * s] / jvs[273 * s]; jvs[598 * s] = -a;
      jvs[602 * s] = jvs[602 * s] + a * jvs[274 * s];
      jvs[632 * s] = jvs[632 * s] + a * jvs[275 * s];
    }
    { const double a = -jvs[599 * s] / jvs[306 * s]; jvs[599 * s] = -a;
      jvs[632 * s] = jvs[632 * s] + a * jvs[307 * s];
      jvs[633 * s] = jvs[633 * s] + a * jvs[308 * s];
    }
    { const double a = -jvs[600 * s] / jvs[310 * s]; jvs[600 * s] = -a;
      jvs[632 * s] = jvs[632 * s] + a * jvs[311 * s];
      jvs[633 * s] = jvs[633 * s] + a * jvs[312 * s];
    }
    { const double a = -jvs[601 * s] / jvs[319 * s]; jvs[601 * s] = -a;
      jvs[604 * s] = jvs[604 * s] + a * jvs[320 * s];
      jvs[620 * s] = jvs[620 * s] + a * jvs[321 * s];
      jvs[630 * s] = jvs[630 * s] + a * jvs[322 * s];
      jvs[632 * s] = jvs[632 * s] + a * jvs[323 * s];
    }
    { const double a = -jvs[602 * s] / jvs[326 * s]; jvs[602 * s] = -a;
      jvs[606 * s] = jvs[606 * s] + a * jvs[327 * s];
      jvs[608 * s] = jvs[608 * s] + a * jvs[328 * s];
      jvs[609 * s] = jvs[609 * s] + a * jvs[329 * s];
      jvs[610 * s] = jvs[610 * s] + a * jvs[330 * s];
      jvs[611 * s] = jvs[611 * s] + a * jvs[331 * s];
      jvs[615 * s] = jvs[615 * s] + a * jvs[332 * s];
      jvs[619 * s] = jvs[619 * s] + a * jvs[333 * s];
      jvs[632 * s] = jvs[632 * s] + a * jvs[334 * s];
      jvs[637 * s] = jvs[637 * s] + a * jvs[335 * s];
    }
    { const double a = -jvs[603 * s] / jvs[337 * s]; jvs[603 * s] = -a;
      jvs[628 * s] = jvs[628 * s] + a * jvs[338 * s];
      jvs[632 * s] = jvs[632 * s] + a * jvs[339 * s];
      jvs[637 * s] = jvs[637 * s] + a * jvs[340 * s];
    }
    { const double a = -jvs[604 * s] / jvs[342 * s]; jvs[604 * s] = -a;
      jvs[630 * s] = jvs[630 * s] + a * jvs[343 * s];
      jvs[633 * s] = jvs[633 * s] + a * jvs[344 * s];
    }
    { const double a = -jvs[605 * s] / jvs[345 * s]; jvs[605 * s] = -a;
      jvs[620 * s] = jvs[620 * s] + a * jvs[346 * s];
      jvs[631 * s] = jvs[631 * s] + a * jvs[347 * s];
      jvs[632 * s] = jvs[632 * s] + a * jvs[348 * s];
      jvs[633 * s] = jvs[633 * s] + a * jvs[349 * s];
    }
    { const double a = -jvs[606 * s] / jvs[350 * s]; jvs[606 * s] = -a;
      jvs[609 * s] = jvs[609 * s] + a * jvs[351 * s];
      jvs[614 * s] = jvs[614 * s] + a * jvs[352 * s];
      jvs[632 * s] = jvs[632 * s] + a * jvs[353 * s];
      jvs[637 * s] = jvs[637 * s] + a * jvs[354 * s];
    }
    { const double a = -jvs[607 * s] / jvs[355 * s]; jvs[607 * s] = -a;
      jvs[626 * s] = jvs[626 * s] + a * jvs[356 * s];
      jvs[627 * s] = jvs[627 * s] + a * jvs[357 * s];
      jvs[632 * s] = jvs[632 * s] + a * jvs[358 * s];
      jvs[635 * s] = jvs[635 * s] + a * jvs[359 * s];
    }
    { const double a = -jvs[608 * s] / jvs[360 * s]; jvs[608 * s] = -a;
      jvs[609 * s] = jvs[609 * s] + a * jvs[361 * s];
      jvs[632 * s] = jvs[632 * s] + a * jvs[362 * s];
      jvs[637 * s] = jvs[637 * s] + a * jvs[363 * s];
    }
    { const double a = -jvs[609 * s] / jvs[366 * s]; jvs[609 * s] = -a;
      jvs[614 * s] = jvs[614 * s] + a * jvs[367 * s];
      jvs[618 * s] = jvs[618 * s] + a * jvs[368 * s];
      jvs[632 * s] = jvs[632 * s] + a * jvs[369 * s];
      jvs[637 * s] = jvs[637 * s] + a * jvs[370 * s];
    }
    { const double a = -jvs[610 * s] / jvs[372 * s]; jvs[610 * s] = -a;
      jvs[611 * s] = jvs[611 * s] + a * jvs[373 * s];
      jvs[632 * s] = jvs[632 * s] + a * jvs[374 * s];
      jvs[637 * s] = jvs[637 * s] + a * jvs[375 * s];
    }
    { const double a = -jvs[611 * s] / jvs[378 * s]; jvs[611 * s] = -a;
      jvs[632 * s] = jvs[632 * s] + a * jvs[379 * s];
      jvs[637 * s] = jvs[637 * s] + a * jvs[380 * s];
    }
    { const double a = -jvs[612 * s] / jvs[383 * s]; jvs[612 * s] = -a;
      jvs[613 * s] = jvs[613 * s] + a * jvs[384 * s];
      jvs[632 * s] = jvs[632 * s] + a * jvs[385 * s];
      jvs[637 * s] = jvs[637 * s] + a * jvs[386 * s];
    }
    { const double a = -jvs[613 * s] / jvs[390 * s]; jvs[613 * s] = -a;
      jvs[632 * s] = jvs[632 * s] + a * jvs[391 * s];
      jvs[637 * s] = jvs[637 * s] + a * jvs[392 * s];
    }
    { const double a = -jvs[614 * s] / jvs[396 * s]; jvs[614 * s] = -a;
      jvs[618 * s] = jvs[618 * s] + a * jvs[397 * s];
      jvs[632 * s] = jvs[632 * s] + a * jvs[398 * s];
      jvs[637 * s] = jvs[637 * s] + a * jvs[399 * s];
    }
    { const double a = -jvs[615 * s] / jvs[400 * s]; jvs[615 * s] = -a;
      jvs[619 * s] = jvs[619 * s] + a * jvs[401 * s];
      jvs[632 * s] = jvs[632 * s] + a * jvs[402 * s];
      jvs[637 * s] = jvs[637 * s] + a * jvs[403 * s];
    }
    { const double a = -jvs[616 * s] / jvs[405 * s]; jvs[616 * s] = -a;
      jvs[617 * s] = jvs[617 * s] + a * jvs[406 * s];
      jvs[632 * s] = jvs[632 * s] + a * jvs[407 * s];
      jvs[637 * s] = jvs[637 * s] + a * jvs[408 * s];
    }
    { const double a = -jvs[617 * s] / jvs[410 * s]; jvs[617 * s] = -a;
      jvs[632 * s] = jvs[632 * s] + a * jvs[411 * s];
      jvs[637 * s] = jvs[637 * s] + a * jvs[412 * s];
    }
    { const double a = -jvs[618 * s] / jvs[418 * s]; jvs[618 * s] = -a;
      jvs[632 * s] = jvs[632 * s] + a * jvs[419 * s];
      jvs[637 * s] = jvs[637 * s] + a * jvs[420 * s];
    }
    { const double a = -jvs[619 * s] / jvs[423 * s]; jvs[619 * s] = -a;
      jvs[624 * s] = jvs[624 * s] + a * jvs[424 * s];
      jvs[625 * s] = jvs[625 * s] + a * jvs[425 * s];
      jvs[632 * s] = jvs[632 * s] + a * jvs[426 * s];
      jvs[637 * s] = jvs[637 * s] + a * jvs[427 * s];
    }
    { const double a = -jvs[620 * s] / jvs[431 * s]; jvs[620 * s] = -a;
      jvs[630 * s] = jvs[630 * s] + a * jvs[432 * s];
      jvs[631 * s] = jvs[631 * s] + a * jvs[433 * s];
      jvs[633 * s] = jvs[633 * s] + a * jvs[434 * s];
      jvs[637 * s] = jvs[637 * s] + a * jvs[435 * s];
    }
    { const double a = -jvs[621 * s] / jvs[446 * s]; jvs[621 * s] = -a;
      jvs[632 * s] = jvs[632 * s] + a * jvs[447 * s];
      jvs[633 * s] = jvs[633 * s] + a * jvs[448 * s];
      jvs[634 * s] = jvs[634 * s] + a * jvs[449 * s];
      jvs[635 * s] = jvs[635 * s] + a * jvs[450 * s];
    }
    { const double a = -jvs[622 * s] / jvs[452 * s]; jvs[622 * s] = -a;
      jvs[627 * s] = jvs[627 * s] + a * jvs[453 * s];
      jvs[631 * s] = jvs[631 * s] + a * jvs[454 * s];
      jvs[632 * s] = jvs[632 * s] + a * jvs[455 * s];
      jvs[633 * s] = jvs[633 * s] + a * jvs[456 * s];
      jvs[637 * s] = jvs[637 * s] + a * jvs[457 * s];
    }
    { const double a = -jvs[623 * s] / jvs[462 * s]; jvs[623 * s] = -a;
      jvs[626 * s] = jvs[626 * s] + a * jvs[463 * s];
      jvs[628 * s] = jvs[628 * s] + a * jvs[464 * s];
      jvs[630 * s] = jvs[630 * s] + a * jvs[465 * s];
      jvs[632 * s] = jvs[632 * s] + a * jvs[466 * s];
      jvs[633 * s] = jvs[633 * s] + a * jvs[467 * s];
      jvs[634 * s] = jvs[634 * s] + a * jvs[468 * s];
    }
    { const double a = -jvs[624 * s] / jvs[470 * s]; jvs[624 * s] = -a;
      jvs[625 * s] = jvs[625 * s] + a * jvs[471 * s];
      jvs[629 * s] = jvs[629 * s] + a * jvs[472 * s];
      jvs[633 * s] = jvs[633 * s] + a * jvs[473 * s];
      jvs[636 * s] = jvs[636 * s] + a * jvs[474 * s];
      jvs[637 * s] = jvs[637 * s] + a * jvs[475 * s];
    }
    { const double a = -jvs[625 * s] / jvs[480 * s]; jvs[625 * s] = -a;
      jvs[629 * s] = jvs[629 * s] + a * jvs[481 * s];
      jvs[632 * s] = jvs[632 * s] + a * jvs[482 * s];
      jvs[633 * s] = jvs[633 * s] + a * jvs[483 * s];
      jvs[636 * s] = jvs[636 * s] + a * jvs[484 * s];
      jvs[637 * s] = jvs[637 * s] + a * jvs[485 * s];
    }
    { const double a = -jvs[626 * s] / jvs[488 * s]; jvs[626 * s] = -a;
      jvs[627 * s] = jvs[627 * s] + a * jvs[489 * s];
      jvs[631 * s] = jvs[631 * s] + a * jvs[490 * s];
      jvs[632 * s] = jvs[632 * s] + a * jvs[491 * s];
      jvs[633 * s] = jvs[633 * s] + a * jvs[492 * s];
      jvs[635 * s] = jvs[635 * s] + a * jvs[493 * s];
    }
    { const double a = -jvs[627 * s] / jvs[494 * s]; jvs[627 * s] = -a;
      jvs[631 * s] = jvs[631 * s] + a * jvs[495 * s];
      jvs[632 * s] = jvs[632 * s] + a * jvs[496 * s];
      jvs[634 * s] = jvs[634 * s] + a * jvs[497 * s];
      jvs[635 * s] = jvs[635 * s] + a * jvs[498 * s];
      jvs[637 * s] = jvs[637 * s] + a * jvs[499 * s];
    }
    { const double a = -jvs[628 * s] / jvs[505 * s]; jvs[628 * s] = -a;
      jvs[631 * s] = jvs[631 * s] + a * jvs[506 * s];
      jvs[632 * s] = jvs[632 * s] + a * jvs[507 * s];
      jvs[633 * s] = jvs[633 * s] + a * jvs[508 * s];
      jvs[634 * s] = jvs[634 * s] + a * jvs[509 * s];
      jvs[635 * s] = jvs[635 * s] + a * jvs[510 * s];
      jvs[636 * s] = jvs[636 * s] + a * jvs[511 * s];
      jvs[637 * s] = jvs[637 * s] + a * jvs[512 * s];
    }
    { const double a = -jvs[629 * s] / jvs[528 * s]; jvs[629 * s] = -a;
      jvs[630 * s] = jvs[630 * s] + a * jvs[529 * s];
      jvs[631 * s] = jvs[631 * s] + a * jvs[530 * s];
      jvs[632 * s] = jvs[632 * s] + a * jvs[531 * s];
      jvs[633 * s] = jvs[633 * s] + a * jvs[532 * s];
      jvs[634 * s] = jvs[634 * s] + a * jvs[533 * s];
      jvs[635 * s] = jvs[635 * s] + a * jvs[534 * s];
      jvs[636 * s] = jvs[636 * s] + a * jvs[535 * s];
      jvs[637 * s] = jvs[637 * s] + a * jvs[536 * s];
    }
    { const double a = -jvs[630 * s] / jvs[555 * s]; jvs[630 * s] = -a;
      jvs[631 * s] = jvs[631 * s] + a * jvs[556 * s];
      jvs[632 * s] = jvs[632 * s] + a * jvs[557 * s];
      jvs[633 * s] = jvs[633 * s] + a * jvs[558 * s];
      jvs[634 * s] = jvs[634 * s] + a * jvs[559 * s];
      jvs[635 * s] = jvs[635 * s] + a * jvs[560 * s];
      jvs[636 * s] = jvs[636 * s] + a * jvs[561 * s];
      jvs[637 * s] = jvs[637 * s] + a * jvs[562 * s];
    }
    { const double a = -jvs[631 * s] / jvs[584 * s]; jvs[631 * s] = -a;
      jvs[632 * s] = jvs[632 * s] + a * jvs[585 * s];
      jvs[633 * s] = jvs[633 * s] + a * jvs[586 * s];
      jvs[634 * s] = jvs[634 * s] + a * jvs[587 * s];
      jvs[635 * s] = jvs[635 * s] + a * jvs[588 * s];
      jvs[636 * s] = jvs[636 * s] + a * jvs[589 * s];
      jvs[637 * s] = jvs[637 * s] + a * jvs[590 * s];
    }
    return 0;
}

KQ_HD KQ_NOINLINE int kqu_decomp_5(double* jvs, long long s)
{
    if (fabs(jvs[657 * s]) < DBL_MIN) return 157;
    { const double a = -jvs[638 * s] / jvs[15 * s]; jvs[638 * s] = -a;
    }
    { const double a = -jvs[639 * s] / jvs[16 * s]; jvs[639 * s] = -a;
    }
    { const double a = -jvs[640 * s] / jvs[302 * s]; jvs[640 * s] = -a;
      jvs[657 * s] = jvs[657 * s] + a * jvs[303 * s];
    }
    { const double a = -jvs[641 * s] / jvs[306 * s]; jvs[641 * s] = -a;
      jvs[656 * s] = jvs[656 * s] + a * jvs[307 * s];
      jvs[657 * s] = jvs[657 * s] + a * jvs[308 * s];
    }
    { const double a = -jvs[642 * s] / jvs[310 * s]; jvs[642 * s] = -a;
      jvs[656 * s] = jvs[656 * s] + a * jvs[311 * s];
      jvs[657 * s] = jvs[657 * s] + a * jvs[312 * s];
    }
    { const double a = -jvs[643 * s] / jvs[342 * s]; jvs[643 * s] = -a;
      jvs[654 * s] = jvs[654 * s] + a * jvs[343 * s];
      jvs[657 * s] = jvs[657 * s] + a * jvs[344 * s];
    }
    { const double a = -jvs[644 * s] / jvs[345 * s]; jvs[644 * s] = -a;
      jvs[645 * s] = jvs[645 * s] + a * jvs[346 * s];
      jvs[655 * s] = jvs[655 * s] + a * jvs[347 * s];
      jvs[656 * s] = jvs[656 * s] + a * jvs[348 * s];
      jvs[657 * s] = jvs[657 * s] + a * jvs[349 * s];
    }
    { const double a = -jvs[645 * s] / jvs[431 * s]; jvs[645 * s] = -a;
      jvs[654 * s] = jvs[654 * s] + a * jvs[432 * s];
      jvs[655 * s] = jvs[655 * s] + a * jvs[433 * s];
      jvs[657 * s] = jvs[657 * s] + a * jvs[434 * s];
      jvs[661 * s] = jvs[661 * s] + a * jvs[435 * s];
    }
    { const double a = -jvs[646 * s] / jvs[438 * s]; jvs[646 * s] = -a;
      jvs[649 * s] = jvs[649 * s] + a * jvs[439 * s];
      jvs[650 * s] = jvs[650 * s] + a * jvs[440 * s];
      jvs[657 * s] = jvs[657 * s] + a * jvs[441 * s];
      jvs[660 * s] = jvs[660 * s] + a * jvs[442 * s];
    }
    { const double a = -jvs[647 * s] / jvs[446 * s]; jvs[647 * s] = -a;
      jvs[656 * s] = jvs[656 * s] + a * jvs[447 * s];
      jvs[657 * s] = jvs[657 * s] + a * jvs[448 * s];
      jvs[658 * s] = jvs[658 * s] + a * jvs[449 * s];
      jvs[659 * s] = jvs[659 * s] + a * jvs[450 * s];
    }
    { const double a = -jvs[648 * s] / jvs[452 * s]; jvs[648 * s] = -a;
      jvs[652 * s] = jvs[652 * s] + a * jvs[453 * s];
      jvs[655 * s] = jvs[655 * s] + a * jvs[454 * s];
      jvs[656 * s] = jvs[656 * s] + a * jvs[455 * s];
      jvs[657 * s] = jvs[657 * s] + a * jvs[456 * s];
      jvs[661 * s] = jvs[661 * s] + a * jvs[457 * s];
    }
    { const double a = -jvs[649 * s] / jvs[470 * s]; jvs[649 * s] = -a;
      jvs[650 * s] = jvs[650 * s] + a * jvs[471 * s];
      jvs[653 * s] = jvs[653 * s] + a * jvs[472 * s];
      jvs[657 * s] = jvs[657 * s] + a * jvs[473 * s];
      jvs[660 * s] = jvs[660 * s] + a * jvs[474 * s];
      jvs[661 * s] = jvs[661 * s] + a * jvs[475 * s];
    }
    { const double a = -jvs[650 * s] / jvs[480 * s]; jvs[650 * s] = -a;
      jvs[653 * s] = jvs[653 * s] + a * jvs[481 * s];
      jvs[656 * s] = jvs[656 * s] + a * jvs[482 * s];
      jvs[657 * s] = jvs[657 * s] + a * jvs[483 * s];
      jvs[660 * s] = jvs[660 * s] + a * jvs[484 * s];
      jvs[661 * s] = jvs[661 * s] + a * jvs[485 * s];
    }
    { const double a = -jvs[651 * s] / jvs[488 * s]; jvs[651 * s] = -a;
      jvs[652 * s] = jvs[652 * s] + a * jvs[489 * s];
      jvs[655 * s] = jvs[655 * s] + a * jvs[490 * s];
      jvs[656 * s] = jvs[656 * s] + a * jvs[491 * s];
      jvs[657 * s] = jvs[657 * s] + a * jvs[492 * s];
      jvs[659 * s] = jvs[659 * s] + a * jvs[493 * s];
    }
    { const double a = -jvs[652 * s] / jvs[494 * s]; jvs[652 * s] = -a;
      jvs[655 * s] = jvs[655 * s] + a * jvs[495 * s];
      jvs[656 * s] = jvs[656 * s] + a * jvs[496 * s];
      jvs[658 * s] = jvs[658 * s] + a * jvs[497 * s];
      jvs[659 * s] = jvs[659 * s] + a * jvs[498 * s];
      jvs[661 * s] = jvs[661 * s] + a * jvs[499 * s];
    }
    { const double a = -jvs[653 * s] / jvs[528 * s]; jvs[653 * s] = -a;
      jvs[654 * s] = jvs[654 * s] + a * jvs[529 * s];
      jvs[655 * s] = jvs[655 * s] + a * jvs[530 * s];
      jvs[656 * s] = jvs[656 * s] + a * jvs[531 * s];
      jvs[657 * s] = jvs[657 * s] + a * jvs[532 * s];
      jvs[658 * s] = jvs[658 * s] + a * jvs[533 * s];
      jvs[659 * s] = jvs[659 * s] + a * jvs[534 * s];
      jvs[660 * s] = jvs[660 * s] + a * jvs[535 * s];
      jvs[661 * s] = jvs[661 * s] + a * jvs[536 * s];
    }
    { const double a = -jvs[654 * s] / jvs[555 * s]; jvs[654 * s] = -a;
      jvs[655 * s] = jvs[655 * s] + a * jvs[556 * s];
      jvs[656 * s] = jvs[656 * s] + a * jvs[557 * s];
      jvs[657 * s] = jvs[657 * s] + a * jvs[558 * s];
      jvs[658 * s] = jvs[658 * s] + a * jvs[559 * s];
      jvs[659 * s] = jvs[659 * s] + a * jvs[560 * s];
      jvs[660 * s] = jvs[660 * s] + a * jvs[561 * s];
      jvs[661 * s] = jvs[661 * s] + a * jvs[562 * s];
    }
    { const double a = -jvs[655 * s] / jvs[584 * s]; jvs[655 * s] = -a;
      jvs[656 * s] = jvs[656 * s] + a * jvs[585 * s];
      jvs[657 * s] = jvs[657 * s] + a * jvs[586 * s];
      jvs[658 * s] = jvs[658 * s] + a * jvs[587 * s];
      jvs[659 * s] = jvs[659 * s] + a * jvs[588 * s];
      jvs[660 * s] = jvs[660 * s] + a * jvs[589 * s];
      jvs[661 * s] = jvs[661 * s] + a * jvs[590 * s];
    }
    { const double a = -jvs[656 * s] / jvs[632 * s]; jvs[656 * s] = -a;
      jvs[657 * s] = jvs[657 * s] + a * jvs[633 * s];
      jvs[658 * s] = jvs[658 * s] + a * jvs[634 * s];
      jvs[659 * s] = jvs[659 * s] + a * jvs[635 * s];
      jvs[660 * s] = jvs[660 * s] + a * jvs[636 * s];
      jvs[661 * s] = jvs[661 * s] + a * jvs[637 * s];
    }
    if (fabs(jvs[669 * s]) < DBL_MIN) return 158;
    { const double a = -jvs[662 * s] / jvs[200 * s]; jvs[662 * s] = -a;
      jvs[669 * s] = jvs[669 * s] + a * jvs[201 * s];
    }
    { const double a = -jvs[663 * s] / jvs[446 * s]; jvs[663 * s] = -a;
      jvs[667 * s] = jvs[667 * s] + a * jvs[447 * s];
      jvs[668 * s] = jvs[668 * s] + a * jvs[448 * s];
      jvs[669 * s] = jvs[669 * s] + a * jvs[449 * s];
      jvs[670 * s] = jvs[670 * s] + a * jvs[450 * s];
    }
    { const double a = -jvs[664 * s] / jvs[494 * s]; jvs[664 * s] = -a;
      jvs[666 * s] = jvs[666 * s] + a * jvs[495 * s];
      jvs[667 * s] = jvs[667 * s] + a * jvs[496 * s];
      jvs[669 * s] = jvs[669 * s] + a * jvs[497 * s];
      jvs[670 * s] = jvs[670 * s] + a * jvs[498 * s];
      jvs[672 * s] = jvs[672 * s] + a * jvs[499 * s];
    }
    { const double a = -jvs[665 * s] / jvs[505 * s]; jvs[665 * s] = -a;
      jvs[666 * s] = jvs[666 * s] + a * jvs[506 * s];
      jvs[667 * s] = jvs[667 * s] + a * jvs[507 * s];
      jvs[668 * s] = jvs[668 * s] + a * jvs[508 * s];
      jvs[669 * s] = jvs[669 * s] + a * jvs[509 * s];
      jvs[670 * s] = jvs[670 * s] + a * jvs[510 * s];
      jvs[671 * s] = jvs[671 * s] + a * jvs[511 * s];
      jvs[672 * s] = jvs[672 * s] + a * jvs[512 * s];
    }
    { const double a = -jvs[666 * s] / jvs[584 * s]; jvs[666 * s] = -a;
      jvs[667 * s] = jvs[667 * s] + a * jvs[585 * s];
      jvs[668 * s] = jvs[668 * s] + a * jvs[586 * s];
      jvs[669 * s] = jvs[669 * s] + a * jvs[587 * s];
      jvs[670 * s] = jvs[670 * s] + a * jvs[588 * s];
      jvs[671 * s] = jvs[671 * s] + a * jvs[589 * s];
      jvs[672 * s] = jvs[672 * s] + a * jvs[590 * s];
    }
    { const double a = -jvs[667 * s] / jvs[632 * s]; jvs[667 * s] = -a;
      jvs[668 * s] = jvs[668 * s] + a * jvs[633 * s];
      jvs[669 * s] = jvs[669 * s] + a * jvs[634 * s];
      jvs[670 * s] = jvs[670 * s] + a * jvs[635 * s];
      jvs[671 * s] = jvs[671 * s] + a * jvs[636 * s];
      jvs[672 * s] = jvs[672 * s] + a * jvs[637 * s];
    }
    { const double a = -jvs[668 * s] / jvs[657 * s]; jvs[668 * s] = -a;
      jvs[669 * s] = jvs[669 * s] + a * jvs[658 * s];
      jvs[670 * s] = jvs[670 * s] + a * jvs[659 * s];
      jvs[671 * s] = jvs[671 * s] + a * jvs[660 * s];
      jvs[672 * s] = jvs[672 * s] + a * jvs[661 * s];
    }
    return 0;
}

KQ_HD KQ_NOINLINE int kqu_decomp_6(double* jvs, long long s)
{
    if (fabs(jvs[685 * s]) < DBL_MIN) return 159;
    { const double a = -jvs[673 * s] / jvs[214 * s]; jvs[673 * s] = -a;
      jvs[685 * s] = jvs[685 * s] + a * jvs[215 * s];
    }
    { const double a = -jvs[674 * s] / jvs[337 * s]; jvs[674 * s] = -a;
      jvs[679 * s] = jvs[679 * s] + a * jvs[338 * s];
      jvs[682 * s] = jvs[682 * s] + a * jvs[339 * s];
      jvs[687 * s] = jvs[687 * s] + a * jvs[340 * s];
    }
    { const double a = -jvs[675 * s] / jvs[446 * s]; jvs[675 * s] = -a;
      jvs[682 * s] = jvs[682 * s] + a * jvs[447 * s];
      jvs[683 * s] = jvs[683 * s] + a * jvs[448 * s];
      jvs[684 * s] = jvs[684 * s] + a * jvs[449 * s];
      jvs[685 * s] = jvs[685 * s] + a * jvs[450 * s];
    }
    { const double a = -jvs[676 * s] / jvs[462 * s]; jvs[676 * s] = -a;
      jvs[677 * s] = jvs[677 * s] + a * jvs[463 * s];
      jvs[679 * s] = jvs[679 * s] + a * jvs[464 * s];
      jvs[680 * s] = jvs[680 * s] + a * jvs[465 * s];
      jvs[682 * s] = jvs[682 * s] + a * jvs[466 * s];
      jvs[683 * s] = jvs[683 * s] + a * jvs[467 * s];
      jvs[684 * s] = jvs[684 * s] + a * jvs[468 * s];
    }
    { const double a = -jvs[677 * s] / jvs[488 * s]; jvs[677 * s] = -a;
      jvs[678 * s] = jvs[678 * s] + a * jvs[489 * s];
      jvs[681 * s] = jvs[681 * s] + a * jvs[490 * s];
      jvs[682 * s] = jvs[682 * s] + a * jvs[491 * s];
      jvs[683 * s] = jvs[683 * s] + a * jvs[492 * s];
      jvs[685 * s] = jvs[685 * s] + a * jvs[493 * s];
    }
    { const double a = -jvs[678 * s] / jvs[494 * s]; jvs[678 * s] = -a;
      jvs[681 * s] = jvs[681 * s] + a * jvs[495 * s];
      jvs[682 * s] = jvs[682 * s] + a * jvs[496 * s];
      jvs[684 * s] = jvs[684 * s] + a * jvs[497 * s];
      jvs[685 * s] = jvs[685 * s] + a * jvs[498 * s];
      jvs[687 * s] = jvs[687 * s] + a * jvs[499 * s];
    }
    { const double a = -jvs[679 * s] / jvs[505 * s]; jvs[679 * s] = -a;
      jvs[681 * s] = jvs[681 * s] + a * jvs[506 * s];
      jvs[682 * s] = jvs[682 * s] + a * jvs[507 * s];
      jvs[683 * s] = jvs[683 * s] + a * jvs[508 * s];
      jvs[684 * s] = jvs[684 * s] + a * jvs[509 * s];
      jvs[685 * s] = jvs[685 * s] + a * jvs[510 * s];
      jvs[686 * s] = jvs[686 * s] + a * jvs[511 * s];
      jvs[687 * s] = jvs[687 * s] + a * jvs[512 * s];
    }
    { const double a = -jvs[680 * s] / jvs[555 * s]; jvs[680 * s] = -a;
      jvs[681 * s] = jvs[681 * s] + a * jvs[556 * s];
      jvs[682 * s] = jvs[682 * s] + a * jvs[557 * s];
      jvs[683 * s] = jvs[683 * s] + a * jvs[558 * s];
      jvs[684 * s] = jvs[684 * s] + a * jvs[559 * s];
      jvs[685 * s] = jvs[685 * s] + a * jvs[560 * s];
      jvs[686 * s] = jvs[686 * s] + a * jvs[561 * s];
      jvs[687 * s] = jvs[687 * s] + a * jvs[562 * s];
    }
    { const double a = -jvs[681 * s] / jvs[584 * s]; jvs[681 * s] = -a;
      jvs[682 * s] = jvs[682 * s] + a * jvs[585 * s];
      jvs[683 * s] = jvs[683 * s] + a * jvs[586 * s];
      jvs[684 * s] = jvs[684 * s] + a * jvs[587 * s];
      jvs[685 * s] = jvs[685 * s] + a * jvs[588 * s];
      jvs[686 * s] = jvs[686 * s] + a * jvs[589 * s];
      jvs[687 * s] = jvs[687 * s] + a * jvs[590 * s];
    }
    { const double a = -jvs[682 * s] / jvs[632 * s]; jvs[682 * s] = -a;
      jvs[683 * s] = jvs[683 * s] + a * jvs[633 * s];
      jvs[684 * s] = jvs[684 * s] + a * jvs[634 * s];
      jvs[685 * s] = jvs[685 * s] + a * jvs[635 * s];
      jvs[686 * s] = jvs[686 * s] + a * jvs[636 * s];
      jvs[687 * s] = jvs[687 * s] + a * jvs[637 * s];
    }
    { const double a = -jvs[683 * s] / jvs[657 * s]; jvs[683 * s] = -a;
      jvs[684 * s] = jvs[684 * s] + a * jvs[658 * s];
      jvs[685 * s] = jvs[685 * s] + a * jvs[659 * s];
      jvs[686 * s] = jvs[686 * s] + a * jvs[660 * s];
      jvs[687 * s] = jvs[687 * s] + a * jvs[661 * s];
    }
    { const double a = -jvs[684 * s] / jvs[669 * s]; jvs[684 * s] = -a;
      jvs[685 * s] = jvs[685 * s] + a * jvs[670 * s];
      jvs[686 * s] = jvs[686 * s] + a * jvs[671 * s];
      jvs[687 * s] = jvs[687 * s] + a * jvs[672 * s];
    }
    if (fabs(jvs[700 * s]) < DBL_MIN) return 160;
    { const double a = -jvs[688 * s] / jvs[15 * s]; jvs[688 * s] = -a;
    }
    { const double a = -jvs[689 * s] / jvs[16 * s]; jvs[689 * s] = -a;
    }
    { const double a = -jvs[690 * s] / jvs[438 * s]; jvs[690 * s] = -a;
      jvs[691 * s] = jvs[691 * s] + a * jvs[439 * s];
      jvs[692 * s] = jvs[692 * s] + a * jvs[440 * s];
      jvs[697 * s] = jvs[697 * s] + a * jvs[441 * s];
      jvs[700 * s] = jvs[700 * s] + a * jvs[442 * s];
    }
    { const double a = -jvs[691 * s] / jvs[470 * s]; jvs[691 * s] = -a;
      jvs[692 * s] = jvs[692 * s] + a * jvs[471 * s];
      jvs[693 * s] = jvs[693 * s] + a * jvs[472 * s];
      jvs[697 * s] = jvs[697 * s] + a * jvs[473 * s];
      jvs[700 * s] = jvs[700 * s] + a * jvs[474 * s];
      jvs[701 * s] = jvs[701 * s] + a * jvs[475 * s];
    }
    { const double a = -jvs[692 * s] / jvs[480 * s]; jvs[692 * s] = -a;
      jvs[693 * s] = jvs[693 * s] + a * jvs[481 * s];
      jvs[696 * s] = jvs[696 * s] + a * jvs[482 * s];
      jvs[697 * s] = jvs[697 * s] + a * jvs[483 * s];
      jvs[700 * s] = jvs[700 * s] + a * jvs[484 * s];
      jvs[701 * s] = jvs[701 * s] + a * jvs[485 * s];
    }
    { const double a = -jvs[693 * s] / jvs[528 * s]; jvs[693 * s] = -a;
      jvs[694 * s] = jvs[694 * s] + a * jvs[529 * s];
      jvs[695 * s] = jvs[695 * s] + a * jvs[530 * s];
      jvs[696 * s] = jvs[696 * s] + a * jvs[531 * s];
      jvs[697 * s] = jvs[697 * s] + a * jvs[532 * s];
      jvs[698 * s] = jvs[698 * s] + a * jvs[533 * s];
      jvs[699 * s] = jvs[699 * s] + a * jvs[534 * s];
      jvs[700 * s] = jvs[700 * s] + a * jvs[535 * s];
      jvs[701 * s] = jvs[701 * s] + a * jvs[536 * s];
    }
    { const double a = -jvs[694 * s] / jvs[555 * s]; jvs[694 * s] = -a;
      jvs[695 * s] = jvs[695 * s] + a * jvs[556 * s];
      jvs[696 * s] = jvs[696 * s] + a * jvs[557 * s];
      jvs[697 * s] = jvs[697 * s] + a * jvs[558 * s];
      jvs[698 * s] = jvs[698 * s] + a * jvs[559 * s];
      jvs[699 * s] = jvs[699 * s] + a * jvs[560 * s];
      jvs[700 * s] = jvs[700 * s] + a * jvs[561 * s];
      jvs[701 * s] = jvs[701 * s] + a * jvs[562 * s];
    }
    { const double a = -jvs[695 * s] / jvs[584 * s]; jvs[695 * s] = -a;
      jvs[696 * s] = jvs[696 * s] + a * jvs[585 * s];
      jvs[697 * s] = jvs[697 * s] + a * jvs[586 * s];
      jvs[698 * s] = jvs[698 * s] + a * jvs[587 * s];
      jvs[699 * s] = jvs[699 * s] + a * jvs[588 * s];
      jvs[700 * s] = jvs[700 * s] + a * jvs[589 * s];
      jvs[701 * s] = jvs[701 * s] + a * jvs[590 * s];
    }
    { const double a = -jvs[696 * s] / jvs[632 * s]; jvs[696 * s] = -a;
      jvs[697 * s] = jvs[697 * s] + a * jvs[633 * s];
      jvs[698 * s] = jvs[698 * s] + a * jvs[634 * s];
      jvs[699 * s] = jvs[699 * s] + a * jvs[635 * s];
      jvs[700 * s] = jvs[700 * s] + a * jvs[636 * s];
      jvs[701 * s] = jvs[701 * s] + a * jvs[637 * s];
    }
    { const double a = -jvs[697 * s] / jvs[657 * s]; jvs[697 * s] = -a;
      jvs[698 * s] = jvs[698 * s] + a * jvs[658 * s];
      jvs[699 * s] = jvs[699 * s] + a * jvs[659 * s];
      jvs[700 * s] = jvs[700 * s] + a * jvs[660 * s];
      jvs[701 * s] = jvs[701 * s] + a * jvs[661 * s];
    }
    { const double a = -jvs[698 * s] / jvs[669 * s]; jvs[698 * s] = -a;
      jvs[699 * s] = jvs[699 * s] + a * jvs[670 * s];
      jvs[700 * s] = jvs[700 * s] + a * jvs[671 * s];
      jvs[701 * s] = jvs[701 * s] + a * jvs[672 * s];
    }
    { const double a = -jvs[699 * s] / jvs[685 * s]; jvs[699 * s] = -a;
      jvs[700 * s] = jvs[700 * s] + a * jvs[686 * s];
      jvs[701 * s] = jvs[701 * s] + a * jvs[687 * s];
    }
    return 0;
}

KQ_HD KQ_NOINLINE int kqu_decomp_7(double* jvs, long long s)
{
    if (fabs(jvs[737 * s]) < DBL_MIN) return 161;
    { const double a = -jvs[702 * s] / jvs[237 * s]; jvs[702 * s] = -a;
      jvs[737 * s] = jvs[737 * s] + a * jvs[238 * s];
    }
    { const double a = -jvs[703 * s] / jvs[241 * s]; jvs[703 * s] = -a;
      jvs[737 * s] = jvs[737 * s] + a * jvs[242 * s];
    }
    { const double a = -jvs[704 * s] / jvs[267 * s]; jvs[704 * s] = -a;
      jvs[737 * s] = jvs[737 * s] + a * jvs[268 * s];
    }
    { const double a = -jvs[705 * s] / jvs[313 * s]; jvs[705 * s] = -a;
      jvs[707 * s] = jvs[707 * s] + a * jvs[314 * s];
      jvs[721 * s] = jvs[721 * s] + a * jvs[315 * s];
      jvs[730 * s] = jvs[730 * s] + a * jvs[316 * s];
    }
    { const double a = -jvs[706 * s] / jvs[337 * s]; jvs[706 * s] = -a;
      jvs[728 * s] = jvs[728 * s] + a * jvs[338 * s];
      jvs[732 * s] = jvs[732 * s] + a * jvs[339 * s];
      jvs[737 * s] = jvs[737 * s] + a * jvs[340 * s];
    }
    { const double a = -jvs[707 * s] / jvs[342 * s]; jvs[707 * s] = -a;
      jvs[730 * s] = jvs[730 * s] + a * jvs[343 * s];
      jvs[733 * s] = jvs[733 * s] + a * jvs[344 * s];
    }
    { const double a = -jvs[708 * s] / jvs[350 * s]; jvs[708 * s] = -a;
      jvs[710 * s] = jvs[710 * s] + a * jvs[351 * s];
      jvs[715 * s] = jvs[715 * s] + a * jvs[352 * s];
      jvs[732 * s] = jvs[732 * s] + a * jvs[353 * s];
      jvs[737 * s] = jvs[737 * s] + a * jvs[354 * s];
    }
    { const double a = -jvs[709 * s] / jvs[360 * s]; jvs[709 * s] = -a;
      jvs[710 * s] = jvs[710 * s] + a * jvs[361 * s];
      jvs[732 * s] = jvs[732 * s] + a * jvs[362 * s];
      jvs[737 * s] = jvs[737 * s] + a * jvs[363 * s];
    }
    { const double a = -jvs[710 * s] / jvs[366 * s]; jvs[710 * s] = -a;
      jvs[715 * s] = jvs[715 * s] + a * jvs[367 * s];
      jvs[719 * s] = jvs[719 * s] + a * jvs[368 * s];
      jvs[732 * s] = jvs[732 * s] + a * jvs[369 * s];
      jvs[737 * s] = jvs[737 * s] + a * jvs[370 * s];
    }
    { const double a = -jvs[711 * s] / jvs[372 * s]; jvs[711 * s] = -a;
      jvs[712 * s] = jvs[712 * s] + a * jvs[373 * s];
      jvs[732 * s] = jvs[732 * s] + a * jvs[374 * s];
      jvs[737 * s] = jvs[737 * s] + a * jvs[375 * s];
    }
    { const double a = -jvs[712 * s] / jvs[378 * s]; jvs[712 * s] = -a;
      jvs[732 * s] = jvs[732 * s] + a * jvs[379 * s];
      jvs[737 * s] = jvs[737 * s] + a * jvs[380 * s];
    }
    { const double a = -jvs[713 * s] / jvs[383 * s]; jvs[713 * s] = -a;
      jvs[714 * s] = jvs[714 * s] + a * jvs[384 * s];
      jvs[732 * s] = jvs[732 * s] + a * jvs[385 * s];
      jvs[737 * s] = jvs[737 * s] + a * jvs[386 * s];
    }
    { const double a = -jvs[714 * s] / jvs[390 * s]; jvs[714 * s] = -a;
      jvs[732 * s] = jvs[732 * s] + a * jvs[391 * s];
      jvs[737 * s] = jvs[737 * s] + a * jvs[392 * s];
    }
    { const double a = -jvs[715 * s] / jvs[396 * s]; jvs[715 * s] = -a;
      jvs[719 * s] = jvs[719 * s] + a * jvs[397 * s];
      jvs[732 * s] = jvs[732 * s] + a * jvs[398 * s];
      jvs[737 * s] = jvs[737 * s] + a * jvs[399 * s];
    }
    { const double a = -jvs[716 * s] / jvs[400 * s]; jvs[716 * s] = -a;
      jvs[720 * s] = jvs[720 * s] + a * jvs[401 * s];
      jvs[732 * s] = jvs[732 * s] + a * jvs[402 * s];
      jvs[737 * s] = jvs[737 * s] + a * jvs[403 * s];
    }
    { const double a = -jvs[717 * s] / jvs[405 * s]; jvs[717 * s] = -a;
      jvs[718 * s] = jvs[718 * s] + a * jvs[406 * s];
      jvs[732 * s] = jvs[732 * s] + a * jvs[407 * s];
      jvs[737 * s] = jvs[737 * s] + a * jvs[408 * s];
    }
    { const double a = -jvs[718 * s] / jvs[410 * s]; jvs[718 * s] = -a;
      jvs[732 * s] = jvs[732 * s] + a * jvs[411 * s];
      jvs[737 * s] = jvs[737 * s] + a * jvs[412 * s];
    }
    { const double a = -jvs[719 * s] / jvs[418 * s]; jvs[719 * s] = -a;
      jvs[732 * s] = jvs[732 * s] + a * jvs[419 * s];
      jvs[737 * s] = jvs[737 * s] + a * jvs[420 * s];
    }
    { const double a = -jvs[720 * s] / jvs[423 * s]; jvs[720 * s] = -a;
      jvs[724 * s] = jvs[724 * s] + a * jvs[424 * s];
      jvs[725 * s] = jvs[725 * s] + a * jvs[425 * s];
      jvs[732 * s] = jvs[732 * s] + a * jvs[426 * s];
      jvs[737 * s] = jvs[737 * s] + a * jvs[427 * s];
    }
    { const double a = -jvs[721 * s] / jvs[431 * s]; jvs[721 * s] = -a;
      jvs[730 * s] = jvs[730 * s] + a * jvs[432 * s];
      jvs[731 * s] = jvs[731 * s] + a * jvs[433 * s];
      jvs[733 * s] = jvs[733 * s] + a * jvs[434 * s];
      jvs[737 * s] = jvs[737 * s] + a * jvs[435 * s];
    }
    { const double a = -jvs[722 * s] / jvs[452 * s]; jvs[722 * s] = -a;
      jvs[727 * s] = jvs[727 * s] + a * jvs[453 * s];
      jvs[731 * s] = jvs[731 * s] + a * jvs[454 * s];
      jvs[732 * s] = jvs[732 * s] + a * jvs[455 * s];
      jvs[733 * s] = jvs[733 * s] + a * jvs[456 * s];
      jvs[737 * s] = jvs[737 * s] + a * jvs[457 * s];
    }
    { const double a = -jvs[723 * s] / jvs[462 * s]; jvs[723 * s] = -a;
      jvs[726 * s] = jvs[726 * s] + a * jvs[463 * s];
      jvs[728 * s] = jvs[728 * s] + a * jvs[464 * s];
      jvs[730 * s] = jvs[730 * s] + a * jvs[465 * s];
      jvs[732 * s] = jvs[732 * s] + a * jvs[466 * s];
      jvs[733 * s] = jvs[733 * s] + a * jvs[467 * s];
      jvs[734 * s] = jvs[734 * s] + a * jvs[468 * s];
    }
    { const double a = -jvs[724 * s] / jvs[470 * s]; jvs[724 * s] = -a;
      jvs[725 * s] = jvs[725 * s] + a * jvs[471 * s];
      jvs[729 * s] = jvs[729 * s] + a * jvs[472 * s];
      jvs[733 * s] = jvs[733 * s] + a * jvs[473 * s];
      jvs[736 * s] = jvs[736 * s] + a * jvs[474 * s];
      jvs[737 * s] = jvs[737 * s] + a * jvs[475 * s];
    }
    { const double a = -jvs[725 * s] / jvs[480 * s]; jvs[725 * s] = -a;
      jvs[729 * s] = jvs[729 * s] + a * jvs[481 * s];
      jvs[732 * s] = jvs[732 * s] + a * jvs[482 * s];
      jvs[733 * s] = jvs[733 * s] + a * jvs[483 * s];
      jvs[736 * s] = jvs[736 * s] + a * jvs[484 * s];
      jvs[737 * s] = jvs[737 * s] + a * jvs[485 * s];
    }
    { const double a = -jvs[726 * s] / jvs[488 * s]; jvs[726 * s] = -a;
      jvs[727 * s] = jvs[727 * s] + a * jvs[489 * s];
      jvs[731 * s] = jvs[731 * s] + a * jvs[490 * s];
      jvs[732 * s] = jvs[732 * s] + a * jvs[491 * s];
      jvs[733 * s] = jvs[733 * s] + a * jvs[492 * s];
      jvs[735 * s] = jvs[735 * s] + a * jvs[493 * s];
    }
    { const double a = -jvs[727 * s] / jvs[494 * s]; jvs[727 * s] = -a;
      jvs[731 * s] = jvs[731 * s] + a * jvs[495 * s];
      jvs[732 * s] = jvs[732 * s] + a * jvs[496 * s];
      jvs[734 * s] = jvs[734 * s] + a * jvs[497 * s];
      jvs[735 * s] = jvs[735 * s] + a * jvs[498 * s];
      jvs[737 * s] = jvs[737 * s] + a * jvs[499 * s];
    }
    { const double a = -jvs[728 * s] / jvs[505 * s]; jvs[728 * s] = -a;
      jvs[731 * s] = jvs[731 * s] + a * jvs[506 * s];
      jvs[732 * s] = jvs[732 * s] + a * jvs[507 * s];
      jvs[733 * s] = jvs[733 * s] + a * jvs[508 * s];
      jvs[734 * s] = jvs[734 * s] + a * jvs[509 * s];
      jvs[735 * s] = jvs[735 * s] + a * jvs[510 * s];
      jvs[736 * s] = jvs[736 * s] + a * jvs[511 * s];
      jvs[737 * s] = jvs[737 * s] + a * jvs[512 * s];
    }
    { const double a = -jvs[729 * s] / jvs[528 * s]; jvs[729 * s] = -a;
      jvs[730 * s] = jvs[730 * s] + a * jvs[529 * s];
      jvs[731 * s] = jvs[731 * s] + a * jvs[530 * s];
      jvs[732 * s] = jvs[732 * s] + a * jvs[531 * s];
      jvs[733 * s] = jvs[733 * s] + a * jvs[532 * s];
      jvs[734 * s] = jvs[734 * s] + a * jvs[533 * s];
      jvs[735 * s] = jvs[735 * s] + a * jvs[534 * s];
      jvs[736 * s] = jvs[736 * s] + a * jvs[535 * s];
      jvs[737 * s] = jvs[737 * s] + a * jvs[536 * s];
    }
    { const double a = -jvs[730 * s] / jvs[555 * s]; jvs[730 * s] = -a;
      jvs[731 * s] = jvs[731 * s] + a * jvs[556 * s];
      jvs[732 * s] = jvs[732 * s] + a * jvs[557 * s];
      jvs[733 * s] = jvs[733 * s] + a * jvs[558 * s];
      jvs[734 * s] = jvs[734 * s] + a * jvs[559 * s];
      jvs[735 * s] = jvs[735 * s] + a * jvs[560 * s];
      jvs[736 * s] = jvs[736 * s] + a * jvs[561 * s];
      jvs[737 * s] = jvs[737 * s] + a * jvs[562 * s];
    }
    { const double a = -jvs[731 * s] / jvs[584 * s]; jvs[731 * s] = -a;
      jvs[732 * s] = jvs[732 * s] + a * jvs[585 * s];
      jvs[733 * s] = jvs[733 * s] + a * jvs[586 * s];
      jvs[734 * s] = jvs[734 * s] + a * jvs[587 * s];
      jvs[735 * s] = jvs[735 * s] + a * jvs[588 * s];
      jvs[736 * s] = jvs[736 * s] + a * jvs[589 * s];
      jvs[737 * s] = jvs[737 * s] + a * jvs[590 * s];
    }
    { const double a = -jvs[732 * s] / jvs[632 * s]; jvs[732 * s] = -a;
      jvs[733 * s] = jvs[733 * s] + a * jvs[633 * s];
      jvs[734 * s] = jvs[734 * s] + a * jvs[634 * s];
      jvs[735 * s] = jvs[735 * s] + a * jvs[635 * s];
      jvs[736 * s] = jvs[736 * s] + a * jvs[636 * s];
      jvs[737 * s] = jvs[737 * s] + a * jvs[637 * s];
    }
    { const double a = -jvs[733 * s] / jvs[657 * s]; jvs[733 * s] = -a;
      jvs[734 * s] = jvs[734 * s] + a * jvs[658 * s];
      jvs[735 * s] = jvs[735 * s] + a * jvs[659 * s];
      jvs[736 * s] = jvs[736 * s] + a * jvs[660 * s];
      jvs[737 * s] = jvs[737 * s] + a * jvs[661 * s];
    }
    { const double a = -jvs[734 * s] / jvs[669 * s]; jvs[734 * s] = -a;
      jvs[735 * s] = jvs[735 * s] + a * jvs[670 * s];
      jvs[736 * s] = jvs[736 * s] + a * jvs[671 * s];
      jvs[737 * s] = jvs[737 * s] + a * jvs[672 * s];
    }
    { const double a = -jvs[735 * s] / jvs[685 * s]; jvs[735 * s] = -a;
      jvs[736 * s] = jvs[736 * s] + a * jvs[686 * s];
      jvs[737 * s] = jvs[737 * s] + a * jvs[687 * s];
    }
    { const double a = -jvs[736 * s] / jvs[700 * s]; jvs[736 * s] = -a;
      jvs[737 * s] = jvs[737 * s] + a * jvs[701 * s];
    }
    return 0;
}

KQ_HD inline int kqu_decomp(double* jvs, long long s)
{
    int rc;
    if ((rc = kqu_decomp_0(jvs, s)) != 0) return rc;
    if ((rc = kqu_decomp_1(jvs, s)) != 0) return rc;
    if ((rc = kqu_decomp_2(jvs, s)) != 0) return rc;
    if ((rc = kqu_decomp_3(jvs, s)) != 0) return rc;
    if ((rc = kqu_decomp_4(jvs, s)) != 0) return rc;
    if ((rc = kqu_decomp_5(jvs, s)) != 0) return rc;
    if ((rc = kqu_decomp_6(jvs, s)) != 0) return rc;
    if ((rc = kqu_decomp_7(jvs, s)) != 0) return rc;
    return 0;
}

KQ_HD KQ_NOINLINE void kqu_solve_f0(const double* jvs, double* x, long long s)
{
    x[8 * s] = x[8 * s] - jvs[8 * s] * x[7 * s];
    x[9 * s] = x[9 * s] - jvs[10 * s] * x[5 * s];
    x[11 * s] = x[11 * s] - jvs[13 * s] * x[6 * s];
    x[17 * s] = x[17 * s] - jvs[20 * s] * x[3 * s];
    x[36 * s] = x[36 * s] - jvs[73 * s] * x[8 * s];
    x[37 * s] = x[37 * s] - jvs[75 * s] * x[12 * s];
    x[38 * s] = x[38 * s] - jvs[77 * s] * x[13 * s];
    x[39 * s] = x[39 * s] - jvs[79 * s] * x[9 * s];
    x[40 * s] = x[40 * s] - jvs[81 * s] * x[10 * s];
    x[41 * s] = x[41 * s] - jvs[83 * s] * x[11 * s];
    x[43 * s] = x[43 * s] - jvs[87 * s] * x[14 * s];
    x[44 * s] = x[44 * s] - jvs[89 * s] * x[15 * s];
    x[45 * s] = x[45 * s] - jvs[91 * s] * x[16 * s];
    x[46 * s] = x[46 * s] - jvs[93 * s] * x[17 * s];
    x[75 * s] = x[75 * s] - jvs[172 * s] * x[74 * s];
    x[77 * s] = x[77 * s] - jvs[177 * s] * x[76 * s];
    x[104 * s] = x[104 * s] - jvs[236 * s] * x[78 * s];
    x[105 * s] = x[105 * s] - jvs[239 * s] * x[93 * s] - jvs[240 * s] * x[104 * s];
    x[106 * s] = x[106 * s] - jvs[243 * s] * x[85 * s];
    x[107 * s] = x[107 * s] - jvs[247 * s] * x[87 * s];
    x[108 * s] = x[108 * s] - jvs[251 * s] * x[1 * s] - jvs[252 * s] * x[107 * s];
    x[110 * s] = x[110 * s] - jvs[258 * s] * x[92 * s];
    x[111 * s] = x[111 * s] - jvs[262 * s] * x[2 * s] - jvs[263 * s] * x[110 * s];
    x[112 * s] = x[112 * s] - jvs[266 * s] * x[94 * s];
    x[114 * s] = x[114 * s] - jvs[272 * s] * x[113 * s];
    x[115 * s] = x[115 * s] - jvs[276 * s] * x[100 * s] - jvs[277 * s] * x[101 * s] - jvs[278 * s] * x[102 * s];
    x[118 * s] = x[118 * s] - jvs[293 * s] * x[83 * s] - jvs[294 * s] * x[116 * s] - jvs[295 * s] * x[117 * s];
    x[119 * s] = x[119 * s] - jvs[301 * s] * x[98 * s];
    x[120 * s] = x[120 * s] - jvs[304 * s] * x[90 * s] - jvs[305 * s] * x[119 * s];
    x[121 * s] = x[121 * s] - jvs[309 * s] * x[91 * s];
    x[123 * s] = x[123 * s] - jvs[317 * s] * x[109 * s] - jvs[318 * s] * x[122 * s];
    x[124 * s] = x[124 * s] - jvs[324 * s] * x[86 * s] - jvs[325 * s] * x[114 * s];
    x[125 * s] = x[125 * s] - jvs[336 * s] * x[73 * s];
    x[126 * s] = x[126 * s] - jvs[341 * s] * x[97 * s];
    x[131 * s] = x[131 * s] - jvs[364 * s] * x[128 * s] - jvs[365 * s] * x[130 * s];
    x[132 * s] = x[132 * s] - jvs[371 * s] * x[112 * s];
    x[133 * s] = x[133 * s] - jvs[376 * s] * x[82 * s] - jvs[377 * s] * x[132 * s];
    x[134 * s] = x[134 * s] - jvs[381 * s] * x[79 * s] - jvs[382 * s] * x[133 * s];
    x[135 * s] = x[135 * s] - jvs[387 * s] * x[132 * s] - jvs[388 * s] * x[133 * s] - jvs[389 * s] * x[134 * s];
    x[136 * s] = x[136 * s] - jvs[393 * s] * x[105 * s] - jvs[394 * s] * x[134 * s] - jvs[395 * s] * x[135 * s];
    x[138 * s] = x[138 * s] - jvs[404 * s] * x[104 * s];
    x[139 * s] = x[139 * s] - jvs[409 * s] * x[138 * s];
}

KQ_HD KQ_NOINLINE void kqu_solve_f1(const double* jvs, double* x, long long s)
{
    x[140 * s] = x[140 * s] - jvs[413 * s] * x[112 * s] - jvs[414 * s] * x[135 * s] - jvs[415 * s] * x[136 * s] - jvs[416 * s] * x[138 * s] - jvs[417 * s] * x[139 * s];
    x[141 * s] = x[141 * s] - jvs[421 * s] * x[89 * s] - jvs[422 * s] * x[137 * s];
    x[142 * s] = x[142 * s] - jvs[428 * s] * x[103 * s] - jvs[429 * s] * x[119 * s] - jvs[430 * s] * x[126 * s];
    x[143 * s] = x[143 * s] - jvs[436 * s] * x[80 * s] - jvs[437 * s] * x[119 * s];
    x[144 * s] = x[144 * s] - jvs[443 * s] * x[12 * s] - jvs[444 * s] * x[13 * s] - jvs[445 * s] * x[99 * s];
    x[145 * s] = x[145 * s] - jvs[451 * s] * x[84 * s];
    x[146 * s] = x[146 * s] - jvs[458 * s] * x[0 * s] - jvs[459 * s] * x[106 * s] - jvs[460 * s] * x[115 * s] - jvs[461 * s] * x[126 * s];
    x[147 * s] = x[147 * s] - jvs[469 * s] * x[143 * s];
    x[148 * s] = x[148 * s] - jvs[476 * s] * x[134 * s] - jvs[477 * s] * x[135 * s] - jvs[478 * s] * x[143 * s] - jvs[479 * s] * x[147 * s];
    x[149 * s] = x[149 * s] - jvs[486 * s] * x[96 * s] - jvs[487 * s] * x[129 * s];
    x[151 * s] = x[151 * s] - jvs[500 * s] * x[125 * s] - jvs[501 * s] * x[129 * s] - jvs[502 * s] * x[144 * s] - jvs[503 * s] * x[149 * s] - jvs[504 * s] * x[150 * s];
    x[152 * s] = x[152 * s] - jvs[513 * s] * x[107 * s] - jvs[514 * s] * x[108 * s] - jvs[515 * s] * x[130 * s] - jvs[516 * s] * x[131 * s] - jvs[517 * s] * x[136 * s] - jvs[518 * s] * x[137 * s] - jvs[519 * s] * x[140 * s] - jvs[520 * s] * x[141 * s] - jvs[521 * s] * x[143 * s] - jvs[522 * s] * x[146 * s] - jvs[523 * s] * x[147 * s] - jvs[524 * s] * x[148 * s] - jvs[525 * s] * x[149 * s] - jvs[526 * s] * x[150 * s] - jvs[527 * s] * x[151 * s];
    x[153 * s] = x[153 * s] - jvs[537 * s] * x[4 * s] - jvs[538 * s] * x[12 * s] - jvs[539 * s] * x[13 * s] - jvs[540 * s] * x[75 * s] - jvs[541 * s] * x[77 * s] - jvs[542 * s] * x[115 * s] - jvs[543 * s] * x[120 * s] - jvs[544 * s] * x[121 * s] - jvs[545 * s] * x[123 * s] - jvs[546 * s] * x[126 * s] - jvs[547 * s] * x[127 * s] - jvs[548 * s] * x[142 * s] - jvs[549 * s] * x[144 * s] - jvs[550 * s] * x[145 * s] - jvs[551 * s] * x[146 * s] - jvs[552 * s] * x[149 * s] - jvs[553 * s] * x[150 * s] - jvs[554 * s] * x[151 * s];
    x[154 * s] = x[154 * s] - jvs[563 * s] * x[81 * s] - jvs[564 * s] * x[104 * s] - jvs[565 * s] * x[105 * s] - jvs[566 * s] * x[112 * s] - jvs[567 * s] * x[119 * s] - jvs[568 * s] * x[132 * s] - jvs[569 * s] * x[133 * s] - jvs[570 * s] * x[136 * s] - jvs[571 * s] * x[137 * s] - jvs[572 * s] * x[138 * s] - jvs[573 * s] * x[139 * s] - jvs[574 * s] * x[140 * s] - jvs[575 * s] * x[141 * s] - jvs[576 * s] * x[142 * s] - jvs[577 * s] * x[145 * s] - jvs[578 * s] * x[147 * s] - jvs[579 * s] * x[148 * s] - jvs[580 * s] * x[149 * s] - jvs[581 * s] * x[150 * s] - jvs[582 * s] * x[152 * s] - jvs[583 * s] * x[153 * s];
    x[155 * s] = x[155 * s] - jvs[591 * s] * x[12 * s] - jvs[592 * s] * x[13 * s] - jvs[593 * s] * x[106 * s] - jvs[594 * s] * x[109 * s] - jvs[595 * s] * x[110 * s] - jvs[596 * s] * x[111 * s] - jvs[597 * s] * x[113 * s] - jvs[598 * s] * x[114 * s] - jvs[599 * s] * x[120 * s] - jvs[600 * s] * x[121 * s] - jvs[601 * s] * x[123 * s] - jvs[602 * s] * x[124 * s] - jvs[603 * s] * x[125 * s] - jvs[604 * s] * x[126 * s] - jvs[605 * s] * x[127 * s] - jvs[606 * s] * x[128 * s] - jvs[607 * s] * x[129 * s] - jvs[608 * s] * x[130 * s] - jvs[609 * s] * x[131 * s] - jvs[610 * s] * x[132 * s] - jvs[611 * s] * x[133 * s] - jvs[612 * s] * x[134 * s] - jvs[613 * s] * x[135 * s] - jvs[614 * s] * x[136 * s] - jvs[615 * s] * x[137 * s] - jvs[616 * s] * x[138 * s] - jvs[617 * s] * x[139 * s] - jvs[618 * s] * x[140 * s] - jvs[619 * s] * x[141 * s] - jvs[620 * s] * x[142 * s] - jvs[621 * s] * x[144 * s] - jvs[622 * s] * x[145 * s] - jvs[623 * s] * x[146 * s] - jvs[624 * s] * x[147 * s] - jvs[625 * s] * x[148 * s] - jvs[626 * s] * x[149 * s] - jvs[627 * s] * x[150 * s] - jvs[628 * s] * x[151 * s] - jvs[629 * s] * x[152 * s] - jvs[630 * s] * x[153 * s] - jvs[631 * s] * x[154 * s];
    x[156 * s] = x[156 * s] - jvs[638 * s] * x[12 * s] - jvs[639 * s] * x[13 * s] - jvs[640 * s] * x[119 * s] - jvs[641 * s] * x[120 * s] - jvs[642 * s] * x[121 * s] - jvs[643 * s] * x[126 * s] - jvs[644 * s] * x[127 * s] - jvs[645 * s] * x[142 * s] - jvs[646 * s] * x[143 * s] - jvs[647 * s] * x[144 * s] - jvs[648 * s] * x[145 * s] - jvs[649 * s] * x[147 * s] - jvs[650 * s] * x[148 * s] - jvs[651 * s] * x[149 * s] - jvs[652 * s] * x[150 * s] - jvs[653 * s] * x[152 * s] - jvs[654 * s] * x[153 * s] - jvs[655 * s] * x[154 * s] - jvs[656 * s] * x[155 * s];
    x[157 * s] = x[157 * s] - jvs[662 * s] * x[88 * s] - jvs[663 * s] * x[144 * s] - jvs[664 * s] * x[150 * s] - jvs[665 * s] * x[151 * s] - jvs[666 * s] * x[154 * s] - jvs[667 * s] * x[155 * s] - jvs[668 * s] * x[156 * s];
    x[158 * s] = x[158 * s] - jvs[673 * s] * x[95 * s] - jvs[674 * s] * x[125 * s] - jvs[675 * s] * x[144 * s] - jvs[676 * s] * x[146 * s] - jvs[677 * s] * x[149 * s] - jvs[678 * s] * x[150 * s] - jvs[679 * s] * x[151 * s] - jvs[680 * s] * x[153 * s] - jvs[681 * s] * x[154 * s] - jvs[682 * s] * x[155 * s] - jvs[683 * s] * x[156 * s] - jvs[684 * s] * x[157 * s];
    x[159 * s] = x[159 * s] - jvs[688 * s] * x[12 * s] - jvs[689 * s] * x[13 * s] - jvs[690 * s] * x[143 * s] - jvs[691 * s] * x[147 * s] - jvs[692 * s] * x[148 * s] - jvs[693 * s] * x[152 * s] - jvs[694 * s] * x[153 * s] - jvs[695 * s] * x[154 * s] - jvs[696 * s] * x[155 * s] - jvs[697 * s] * x[156 * s] - jvs[698 * s] * x[157 * s] - jvs[699 * s] * x[158 * s];
}

KQ_HD KQ_NOINLINE void kqu_solve_f2(const double* jvs, double* x, long long s)
{
    x[160 * s] = x[160 * s] - jvs[702 * s] * x[104 * s] - jvs[703 * s] * x[105 * s] - jvs[704 * s] * x[112 * s] - jvs[705 * s] * x[122 * s] - jvs[706 * s] * x[125 * s] - jvs[707 * s] * x[126 * s] - jvs[708 * s] * x[128 * s] - jvs[709 * s] * x[130 * s] - jvs[710 * s] * x[131 * s] - jvs[711 * s] * x[132 * s] - jvs[712 * s] * x[133 * s] - jvs[713 * s] * x[134 * s] - jvs[714 * s] * x[135 * s] - jvs[715 * s] * x[136 * s] - jvs[716 * s] * x[137 * s] - jvs[717 * s] * x[138 * s] - jvs[718 * s] * x[139 * s] - jvs[719 * s] * x[140 * s] - jvs[720 * s] * x[141 * s] - jvs[721 * s] * x[142 * s] - jvs[722 * s] * x[145 * s] - jvs[723 * s] * x[146 * s] - jvs[724 * s] * x[147 * s] - jvs[725 * s] * x[148 * s] - jvs[726 * s] * x[149 * s] - jvs[727 * s] * x[150 * s] - jvs[728 * s] * x[151 * s] - jvs[729 * s] * x[152 * s] - jvs[730 * s] * x[153 * s] - jvs[731 * s] * x[154 * s] - jvs[732 * s] * x[155 * s] - jvs[733 * s] * x[156 * s] - jvs[734 * s] * x[157 * s] - jvs[735 * s] * x[158 * s] - jvs[736 * s] * x[159 * s];
}

KQ_HD KQ_NOINLINE void kqu_solve_b0(const double* jvs, double* x, long long s)
{
    x[160 * s] = (x[160 * s]) / jvs[737 * s];
    x[159 * s] = (x[159 * s] - jvs[701 * s] * x[160 * s]) / jvs[700 * s];
    x[158 * s] = (x[158 * s] - jvs[686 * s] * x[159 * s] - jvs[687 * s] * x[160 * s]) / jvs[685 * s];
    x[157 * s] = (x[157 * s] - jvs[670 * s] * x[158 * s] - jvs[671 * s] * x[159 * s] - jvs[672 * s] * x[160 * s]) / jvs[669 * s];
    x[156 * s] = (x[156 * s] - jvs[658 * s] * x[157 * s] - jvs[659 * s] * x[158 * s] - jvs[660 * s] * x[159 * s] - jvs[661 * s] * x[160 * s]) / jvs[657 * s];
    x[155 * s] = (x[155 * s] - jvs[633 * s] * x[156 * s] - jvs[634 * s] * x[157 * s] - jvs[635 * s] * x[158 * s] - jvs[636 * s] * x[159 * s] - jvs[637 * s] * x[160 * s]) / jvs[632 * s];
    x[154 * s] = (x[154 * s] - jvs[585 * s] * x[155 * s] - jvs[586 * s] * x[156 * s] - jvs[587 * s] * x[157 * s] - jvs[588 * s] * x[158 * s] - jvs[589 * s] * x[159 * s] - jvs[590 * s] * x[160 * s]) / jvs[584 * s];
    x[153 * s] = (x[153 * s] - jvs[556 * s] * x[154 * s] - jvs[557 * s] * x[155 * s] - jvs[558 * s] * x[156 * s] - jvs[559 * s] * x[157 * s] - jvs[560 * s] * x[158 * s] - jvs[561 * s] * x[159 * s] - jvs[562 * s] * x[160 * s]) / jvs[555 * s];
    x[152 * s] = (x[152 * s] - jvs[529 * s] * x[153 * s] - jvs[530 * s] * x[154 * s] - jvs[531 * s] * x[155 * s] - jvs[532 * s] * x[156 * s] - jvs[533 * s] * x[157 * s] - jvs[534 * s] * x[158 * s] - jvs[535 * s] * x[159 * s] - jvs[536 * s] * x[160 * s]) / jvs[528 * s];
    x[151 * s] = (x[151 * s] - jvs[506 * s] * x[154 * s] - jvs[507 * s] * x[155 * s] - jvs[508 * s] * x[156 * s] - jvs[509 * s] * x[157 * s] - jvs[510 * s] * x[158 * s] - jvs[511 * s] * x[159 * s] - jvs[512 * s] * x[160 * s]) / jvs[505 * s];
    x[150 * s] = (x[150 * s] - jvs[495 * s] * x[154 * s] - jvs[496 * s] * x[155 * s] - jvs[497 * s] * x[157 * s] - jvs[498 * s] * x[158 * s] - jvs[499 * s] * x[160 * s]) / jvs[494 * s];
    x[149 * s] = (x[149 * s] - jvs[489 * s] * x[150 * s] - jvs[490 * s] * x[154 * s] - jvs[491 * s] * x[155 * s] - jvs[492 * s] * x[156 * s] - jvs[493 * s] * x[158 * s]) / jvs[488 * s];
    x[148 * s] = (x[148 * s] - jvs[481 * s] * x[152 * s] - jvs[482 * s] * x[155 * s] - jvs[483 * s] * x[156 * s] - jvs[484 * s] * x[159 * s] - jvs[485 * s] * x[160 * s]) / jvs[480 * s];
    x[147 * s] = (x[147 * s] - jvs[471 * s] * x[148 * s] - jvs[472 * s] * x[152 * s] - jvs[473 * s] * x[156 * s] - jvs[474 * s] * x[159 * s] - jvs[475 * s] * x[160 * s]) / jvs[470 * s];
    x[146 * s] = (x[146 * s] - jvs[463 * s] * x[149 * s] - jvs[464 * s] * x[151 * s] - jvs[465 * s] * x[153 * s] - jvs[466 * s] * x[155 * s] - jvs[467 * s] * x[156 * s] - jvs[468 * s] * x[157 * s]) / jvs[462 * s];
    x[145 * s] = (x[145 * s] - jvs[453 * s] * x[150 * s] - jvs[454 * s] * x[154 * s] - jvs[455 * s] * x[155 * s] - jvs[456 * s] * x[156 * s] - jvs[457 * s] * x[160 * s]) / jvs[452 * s];
    x[144 * s] = (x[144 * s] - jvs[447 * s] * x[155 * s] - jvs[448 * s] * x[156 * s] - jvs[449 * s] * x[157 * s] - jvs[450 * s] * x[158 * s]) / jvs[446 * s];
    x[143 * s] = (x[143 * s] - jvs[439 * s] * x[147 * s] - jvs[440 * s] * x[148 * s] - jvs[441 * s] * x[156 * s] - jvs[442 * s] * x[159 * s]) / jvs[438 * s];
    x[142 * s] = (x[142 * s] - jvs[432 * s] * x[153 * s] - jvs[433 * s] * x[154 * s] - jvs[434 * s] * x[156 * s] - jvs[435 * s] * x[160 * s]) / jvs[431 * s];
    x[141 * s] = (x[141 * s] - jvs[424 * s] * x[147 * s] - jvs[425 * s] * x[148 * s] - jvs[426 * s] * x[155 * s] - jvs[427 * s] * x[160 * s]) / jvs[423 * s];
    x[140 * s] = (x[140 * s] - jvs[419 * s] * x[155 * s] - jvs[420 * s] * x[160 * s]) / jvs[418 * s];
    x[139 * s] = (x[139 * s] - jvs[411 * s] * x[155 * s] - jvs[412 * s] * x[160 * s]) / jvs[410 * s];
    x[138 * s] = (x[138 * s] - jvs[406 * s] * x[139 * s] - jvs[407 * s] * x[155 * s] - jvs[408 * s] * x[160 * s]) / jvs[405 * s];
    x[137 * s] = (x[137 * s] - jvs[401 * s] * x[141 * s] - jvs[402 * s] * x[155 * s] - jvs[403 * s] * x[160 * s]) / jvs[400 * s];
    x[136 * s] = (x[136 * s] - jvs[397 * s] * x[140 * s] - jvs[398 * s] * x[155 * s] - jvs[399 * s] * x[160 * s]) / jvs[396 * s];
    x[135 * s] = (x[135 * s] - jvs[391 * s] * x[155 * s] - jvs[392 * s] * x[160 * s]) / jvs[390 * s];
    x[134 * s] = (x[134 * s] - jvs[384 * s] * x[135 * s] - jvs[385 * s] * x[155 * s] - jvs[386 * s] * x[160 * s]) / jvs[383 * s];
    x[133 * s] = (x[133 * s] - jvs[379 * s] * x[155 * s] - jvs[380 * s] * x[160 * s]) / jvs[378 * s];
    x[132 * s] = (x[132 * s] - jvs[373 * s] * x[133 * s] - jvs[374 * s] * x[155 * s] - jvs[375 * s] * x[160 * s]) / jvs[372 * s];
    x[131 * s] = (x[131 * s] - jvs[367 * s] * x[136 * s] - jvs[368 * s] * x[140 * s] - jvs[369 * s] * x[155 * s] - jvs[370 * s] * x[160 * s]) / jvs[366 * s];
    x[130 * s] = (x[130 * s] - jvs[361 * s] * x[131 * s] - jvs[362 * s] * x[155 * s] - jvs[363 * s] * x[160 * s]) / jvs[360 * s];
    x[129 * s] = (x[129 * s] - jvs[356 * s] * x[149 * s] - jvs[357 * s] * x[150 * s] - jvs[358 * s] * x[155 * s] - jvs[359 * s] * x[158 * s]) / jvs[355 * s];
    x[128 * s] = (x[128 * s] - jvs[351 * s] * x[131 * s] - jvs[352 * s] * x[136 * s] - jvs[353 * s] * x[155 * s] - jvs[354 * s] * x[160 * s]) / jvs[350 * s];
    x[127 * s] = (x[127 * s] - jvs[346 * s] * x[142 * s] - jvs[347 * s] * x[154 * s] - jvs[348 * s] * x[155 * s] - jvs[349 * s] * x[156 * s]) / jvs[345 * s];
    x[126 * s] = (x[126 * s] - jvs[343 * s] * x[153 * s] - jvs[344 * s] * x[156 * s]) / jvs[342 * s];
    x[125 * s] = (x[125 * s] - jvs[338 * s] * x[151 * s] - jvs[339 * s] * x[155 * s] - jvs[340 * s] * x[160 * s]) / jvs[337 * s];
    x[124 * s] = (x[124 * s] - jvs[327 * s] * x[128 * s] - jvs[328 * s] * x[130 * s] - jvs[329 * s] * x[131 * s] - jvs[330 * s] * x[132 * s] - jvs[331 * s] * x[133 * s] - jvs[332 * s] * x[137 * s] - jvs[333 * s] * x[141 * s] - jvs[334 * s] * x[155 * s] - jvs[335 * s] * x[160 * s]) / jvs[326 * s];
    x[123 * s] = (x[123 * s] - jvs[320 * s] * x[126 * s] - jvs[321 * s] * x[142 * s] - jvs[322 * s] * x[153 * s] - jvs[323 * s] * x[155 * s]) / jvs[319 * s];
    x[122 * s] = (x[122 * s] - jvs[314 * s] * x[126 * s] - jvs[315 * s] * x[142 * s] - jvs[316 * s] * x[153 * s]) / jvs[313 * s];
    x[121 * s] = (x[121 * s] - jvs[311 * s] * x[155 * s] - jvs[312 * s] * x[156 * s]) / jvs[310 * s];
    x[120 * s] = (x[120 * s] - jvs[307 * s] * x[155 * s] - jvs[308 * s] * x[156 * s]) / jvs[306 * s];
    x[119 * s] = (x[119 * s] - jvs[303 * s] * x[156 * s]) / jvs[302 * s];
}

KQ_HD KQ_NOINLINE void kqu_solve_b1(const double* jvs, double* x, long long s)
{
    x[118 * s] = (x[118 * s] - jvs[297 * s] * x[152 * s] - jvs[298 * s] * x[156 * s] - jvs[299 * s] * x[159 * s] - jvs[300 * s] * x[160 * s]) / jvs[296 * s];
    x[117 * s] = (x[117 * s] - jvs[288 * s] * x[118 * s] - jvs[289 * s] * x[152 * s] - jvs[290 * s] * x[156 * s] - jvs[291 * s] * x[159 * s] - jvs[292 * s] * x[160 * s]) / jvs[287 * s];
    x[116 * s] = (x[116 * s] - jvs[283 * s] * x[117 * s] - jvs[284 * s] * x[118 * s] - jvs[285 * s] * x[152 * s] - jvs[286 * s] * x[160 * s]) / jvs[282 * s];
    x[115 * s] = (x[115 * s] - jvs[280 * s] * x[146 * s] - jvs[281 * s] * x[153 * s]) / jvs[279 * s];
    x[114 * s] = (x[114 * s] - jvs[274 * s] * x[124 * s] - jvs[275 * s] * x[155 * s]) / jvs[273 * s];
    x[113 * s] = (x[113 * s] - jvs[270 * s] * x[114 * s] - jvs[271 * s] * x[155 * s]) / jvs[269 * s];
    x[112 * s] = (x[112 * s] - jvs[268 * s] * x[160 * s]) / jvs[267 * s];
    x[111 * s] = (x[111 * s] - jvs[265 * s] * x[155 * s]) / jvs[264 * s];
    x[110 * s] = (x[110 * s] - jvs[260 * s] * x[111 * s] - jvs[261 * s] * x[155 * s]) / jvs[259 * s];
    x[109 * s] = (x[109 * s] - jvs[256 * s] * x[123 * s] - jvs[257 * s] * x[155 * s]) / jvs[255 * s];
    x[108 * s] = (x[108 * s] - jvs[254 * s] * x[152 * s]) / jvs[253 * s];
    x[107 * s] = (x[107 * s] - jvs[249 * s] * x[108 * s] - jvs[250 * s] * x[152 * s]) / jvs[248 * s];
    x[106 * s] = (x[106 * s] - jvs[245 * s] * x[146 * s] - jvs[246 * s] * x[155 * s]) / jvs[244 * s];
    x[105 * s] = (x[105 * s] - jvs[242 * s] * x[160 * s]) / jvs[241 * s];
    x[104 * s] = (x[104 * s] - jvs[238 * s] * x[160 * s]) / jvs[237 * s];
    x[103 * s] = (x[103 * s] - jvs[232 * s] * x[119 * s] - jvs[233 * s] * x[126 * s] - jvs[234 * s] * x[156 * s] - jvs[235 * s] * x[160 * s]) / jvs[231 * s];
    x[102 * s] = (x[102 * s] - jvs[229 * s] * x[115 * s] - jvs[230 * s] * x[153 * s]) / jvs[228 * s];
    x[101 * s] = (x[101 * s] - jvs[227 * s] * x[115 * s]) / jvs[226 * s];
    x[100 * s] = (x[100 * s] - jvs[225 * s] * x[115 * s]) / jvs[224 * s];
    x[99 * s] = (x[99 * s] - jvs[223 * s] * x[144 * s]) / jvs[222 * s];
    x[98 * s] = (x[98 * s] - jvs[221 * s] * x[119 * s]) / jvs[220 * s];
    x[97 * s] = (x[97 * s] - jvs[219 * s] * x[126 * s]) / jvs[218 * s];
    x[96 * s] = (x[96 * s] - jvs[217 * s] * x[149 * s]) / jvs[216 * s];
    x[95 * s] = (x[95 * s] - jvs[215 * s] * x[158 * s]) / jvs[214 * s];
    x[94 * s] = (x[94 * s] - jvs[213 * s] * x[112 * s]) / jvs[212 * s];
    x[93 * s] = (x[93 * s] - jvs[211 * s] * x[105 * s]) / jvs[210 * s];
    x[92 * s] = (x[92 * s] - jvs[209 * s] * x[110 * s]) / jvs[208 * s];
    x[91 * s] = (x[91 * s] - jvs[207 * s] * x[121 * s]) / jvs[206 * s];
    x[90 * s] = (x[90 * s] - jvs[205 * s] * x[120 * s]) / jvs[204 * s];
    x[89 * s] = (x[89 * s] - jvs[203 * s] * x[141 * s]) / jvs[202 * s];
    x[88 * s] = (x[88 * s] - jvs[201 * s] * x[157 * s]) / jvs[200 * s];
    x[87 * s] = (x[87 * s] - jvs[199 * s] * x[107 * s]) / jvs[198 * s];
    x[86 * s] = (x[86 * s] - jvs[197 * s] * x[124 * s]) / jvs[196 * s];
    x[85 * s] = (x[85 * s] - jvs[195 * s] * x[106 * s]) / jvs[194 * s];
    x[84 * s] = (x[84 * s] - jvs[193 * s] * x[145 * s]) / jvs[192 * s];
    x[83 * s] = (x[83 * s] - jvs[191 * s] * x[118 * s]) / jvs[190 * s];
    x[82 * s] = (x[82 * s] - jvs[189 * s] * x[133 * s]) / jvs[188 * s];
    x[81 * s] = (x[81 * s] - jvs[187 * s] * x[154 * s]) / jvs[186 * s];
    x[80 * s] = (x[80 * s] - jvs[185 * s] * x[143 * s]) / jvs[184 * s];
    x[79 * s] = (x[79 * s] - jvs[183 * s] * x[134 * s]) / jvs[182 * s];
    x[78 * s] = (x[78 * s] - jvs[181 * s] * x[104 * s]) / jvs[180 * s];
    x[77 * s] = (x[77 * s] - jvs[179 * s] * x[153 * s]) / jvs[178 * s];
    x[76 * s] = (x[76 * s] - jvs[176 * s] * x[77 * s]) / jvs[175 * s];
    x[75 * s] = (x[75 * s] - jvs[174 * s] * x[153 * s]) / jvs[173 * s];
    x[74 * s] = (x[74 * s] - jvs[171 * s] * x[75 * s]) / jvs[170 * s];
    x[73 * s] = (x[73 * s] - jvs[169 * s] * x[125 * s]) / jvs[168 * s];
    x[72 * s] = (x[72 * s] - jvs[167 * s] * x[119 * s]) / jvs[166 * s];
    x[71 * s] = (x[71 * s] - jvs[165 * s] * x[126 * s]) / jvs[164 * s];
    x[70 * s] = (x[70 * s] - jvs[161 * s] * x[116 * s] - jvs[162 * s] * x[117 * s] - jvs[163 * s] * x[118 * s]) / jvs[160 * s];
    x[69 * s] = (x[69 * s] - jvs[158 * s] * x[138 * s] - jvs[159 * s] * x[139 * s]) / jvs[157 * s];
    x[68 * s] = (x[68 * s] - jvs[156 * s] * x[104 * s]) / jvs[155 * s];
    x[67 * s] = (x[67 * s] - jvs[153 * s] * x[150 * s] - jvs[154 * s] * x[154 * s]) / jvs[152 * s];
    x[66 * s] = (x[66 * s] - jvs[149 * s] * x[143 * s] - jvs[150 * s] * x[147 * s] - jvs[151 * s] * x[148 * s]) / jvs[148 * s];
    x[65 * s] = (x[65 * s] - jvs[146 * s] * x[134 * s] - jvs[147 * s] * x[135 * s]) / jvs[145 * s];
    x[64 * s] = (x[64 * s] - jvs[143 * s] * x[132 * s] - jvs[144 * s] * x[133 * s]) / jvs[142 * s];
    x[63 * s] = (x[63 * s] - jvs[139 * s] * x[128 * s] - jvs[140 * s] * x[130 * s] - jvs[141 * s] * x[131 * s]) / jvs[138 * s];
    x[62 * s] = (x[62 * s] - jvs[136 * s] * x[136 * s] - jvs[137 * s] * x[140 * s]) / jvs[135 * s];
    x[61 * s] = (x[61 * s] - jvs[132 * s] * x[75 * s] - jvs[133 * s] * x[77 * s] - jvs[134 * s] * x[153 * s]) / jvs[131 * s];
    x[60 * s] = (x[60 * s] - jvs[130 * s] * x[61 * s]) / jvs[129 * s];
    x[59 * s] = (x[59 * s] - jvs[127 * s] * x[75 * s] - jvs[128 * s] * x[77 * s]) / jvs[126 * s];
    x[58 * s] = (x[58 * s] - jvs[125 * s] * x[59 * s]) / jvs[124 * s];
    x[57 * s] = (x[57 * s] - jvs[123 * s] * x[77 * s]) / jvs[122 * s];
    x[56 * s] = (x[56 * s] - jvs[121 * s] * x[75 * s]) / jvs[120 * s];
    x[55 * s] = (x[55 * s] - jvs[117 * s] * x[101 * s] - jvs[118 * s] * x[102 * s] - jvs[119 * s] * x[115 * s]) / jvs[116 * s];
    x[54 * s] = (x[54 * s] - jvs[115 * s] * x[55 * s]) / jvs[114 * s];
    x[53 * s] = (x[53 * s] - jvs[113 * s] * x[102 * s]) / jvs[112 * s];
    x[52 * s] = (x[52 * s] - jvs[109 * s] * x[115 * s] - jvs[110 * s] * x[146 * s] - jvs[111 * s] * x[153 * s]) / jvs[108 * s];
    x[51 * s] = (x[51 * s] - jvs[106 * s] * x[52 * s] - jvs[107 * s] * x[101 * s]) / jvs[105 * s];
    x[50 * s] = (x[50 * s] - jvs[104 * s] * x[115 * s]) / jvs[103 * s];
    x[49 * s] = (x[49 * s] - jvs[101 * s] * x[129 * s] - jvs[102 * s] * x[149 * s]) / jvs[100 * s];
    x[48 * s] = (x[48 * s] - jvs[98 * s] * x[125 * s] - jvs[99 * s] * x[151 * s]) / jvs[97 * s];
    x[47 * s] = (x[47 * s] - jvs[96 * s] * x[158 * s]) / jvs[95 * s];
    x[46 * s] = (x[46 * s]) / jvs[94 * s];
    x[45 * s] = (x[45 * s]) / jvs[92 * s];
    x[44 * s] = (x[44 * s]) / jvs[90 * s];
    x[43 * s] = (x[43 * s]) / jvs[88 * s];
    x[42 * s] = (x[42 * s] - jvs[86 * s] * x[155 * s]) / jvs[85 * s];
    x[41 * s] = (x[41 * s]) / jvs[84 * s];
    x[40 * s] = (x[40 * s]) / jvs[82 * s];
    x[39 * s] = (x[39 * s]) / jvs[80 * s];
    x[38 * s] = (x[38 * s]) / jvs[78 * s];
    x[37 * s] = (x[37 * s]) / jvs[76 * s];
    x[36 * s] = (x[36 * s]) / jvs[74 * s];
    x[35 * s] = (x[35 * s] - jvs[72 * s] * x[111 * s]) / jvs[71 * s];
}

KQ_HD KQ_NOINLINE void kqu_solve_b2(const double* jvs, double* x, long long s)
{
    x[34 * s] = (x[34 * s] - jvs[70 * s] * x[108 * s]) / jvs[69 * s];
    x[33 * s] = (x[33 * s] - jvs[68 * s] * x[146 * s]) / jvs[67 * s];
    x[32 * s] = (x[32 * s] - jvs[66 * s] * x[160 * s]) / jvs[65 * s];
    x[31 * s] = (x[31 * s] - jvs[64 * s] * x[112 * s]) / jvs[63 * s];
    x[30 * s] = (x[30 * s] - jvs[62 * s] * x[105 * s]) / jvs[61 * s];
    x[29 * s] = (x[29 * s] - jvs[60 * s] * x[110 * s]) / jvs[59 * s];
    x[28 * s] = (x[28 * s] - jvs[56 * s] * x[109 * s] - jvs[57 * s] * x[123 * s] - jvs[58 * s] * x[153 * s]) / jvs[55 * s];
    x[27 * s] = (x[27 * s] - jvs[54 * s] * x[121 * s]) / jvs[53 * s];
    x[26 * s] = (x[26 * s] - jvs[52 * s] * x[120 * s]) / jvs[51 * s];
    x[25 * s] = (x[25 * s] - jvs[49 * s] * x[137 * s] - jvs[50 * s] * x[141 * s]) / jvs[48 * s];
    x[24 * s] = (x[24 * s] - jvs[47 * s] * x[157 * s]) / jvs[46 * s];
    x[23 * s] = (x[23 * s] - jvs[45 * s] * x[145 * s]) / jvs[44 * s];
    x[22 * s] = (x[22 * s] - jvs[43 * s] * x[107 * s]) / jvs[42 * s];
    x[21 * s] = (x[21 * s] - jvs[39 * s] * x[130 * s] - jvs[40 * s] * x[131 * s] - jvs[41 * s] * x[160 * s]) / jvs[38 * s];
    x[20 * s] = (x[20 * s] - jvs[34 * s] * x[21 * s] - jvs[35 * s] * x[113 * s] - jvs[36 * s] * x[114 * s] - jvs[37 * s] * x[124 * s]) / jvs[33 * s];
    x[19 * s] = (x[19 * s] - jvs[32 * s] * x[106 * s]) / jvs[31 * s];
    x[18 * s] = (x[18 * s] - jvs[23 * s] * x[103 * s] - jvs[24 * s] * x[122 * s] - jvs[25 * s] * x[127 * s] - jvs[26 * s] * x[142 * s] - jvs[27 * s] * x[144 * s] - jvs[28 * s] * x[147 * s] - jvs[29 * s] * x[156 * s] - jvs[30 * s] * x[159 * s]) / jvs[22 * s];
    x[17 * s] = (x[17 * s]) / jvs[21 * s];
    x[16 * s] = (x[16 * s]) / jvs[19 * s];
    x[15 * s] = (x[15 * s]) / jvs[18 * s];
    x[14 * s] = (x[14 * s]) / jvs[17 * s];
    x[13 * s] = (x[13 * s]) / jvs[16 * s];
    x[12 * s] = (x[12 * s]) / jvs[15 * s];
    x[11 * s] = (x[11 * s]) / jvs[14 * s];
    x[10 * s] = (x[10 * s]) / jvs[12 * s];
    x[9 * s] = (x[9 * s]) / jvs[11 * s];
    x[8 * s] = (x[8 * s]) / jvs[9 * s];
    x[7 * s] = (x[7 * s]) / jvs[7 * s];
    x[6 * s] = (x[6 * s]) / jvs[6 * s];
    x[5 * s] = (x[5 * s]) / jvs[5 * s];
    x[4 * s] = (x[4 * s]) / jvs[4 * s];
    x[3 * s] = (x[3 * s]) / jvs[3 * s];
    x[2 * s] = (x[2 * s]) / jvs[2 * s];
    x[1 * s] = (x[1 * s]) / jvs[1 * s];
    x[0 * s] = (x[0 * s]) / jvs[0 * s];
}

KQ_HD inline void kqu_solve(const double* jvs, double* x, long long s)
{
    kqu_solve_f0(jvs, x, s);
    kqu_solve_f1(jvs, x, s);
    kqu_solve_f2(jvs, x, s);
    kqu_solve_b0(jvs, x, s);
    kqu_solve_b1(jvs, x, s);
    kqu_solve_b2(jvs, x, s);
}
