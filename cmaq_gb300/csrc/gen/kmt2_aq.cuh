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

KQ_HD KQ_NOINLINE void kq_rates_once(const Cell& c, const double* v, const double* f, double* r)
{
    (void)v;
    (void)f;
    r[0 * KQ_S] = kq_kmtf(c, 0x1.c28f5c28f5c29p-4, 0x1.ad7f29abcaf48p-17, 0x1.004189374bc6ap+6);
    r[1 * KQ_S] = kq_kmtf(c, 0x1.63886594af4f1p-4, 0x1.baeb22f9294c3p-17, 0x1.f81a9fbe76c8bp+5);
    r[2 * KQ_S] = kq_kmtf(c, 0x1.3a92a30553261p-13, 0x1.040bfe3b03e21p-16, 0x1.60147ae147ae1p+5);
    r[3 * KQ_S] = kq_kmtf(c, 0x1.74bc6a7ef9db2p-4, 0x1.81e03f705857bp-16, 0x1.107ef9db22d0ep+4);
    r[4 * KQ_S] = kq_kmtf(c, 0x1.39c0ebedfa440p-3, 0x1.e9e50b87f37efp-17, 0x1.101eb851eb852p+5);
    r[5 * KQ_S] = kq_kmtf(c, 0x1.999999999999ap-4, 0x1.f09b082ea2aacp-17, 0x1.7ffbe76c8b439p+5);
    r[6 * KQ_S] = kq_kmtf(c, 0x1.77318fc504817p-6, 0x1.00b0ffe7ac4c2p-16, 0x1.7033333333333p+5);
    r[7 * KQ_S] = kq_kmtf(c, 0x1.bae46cfc829d0p-8, 0x1.b79024a5d1b64p-17, 0x1.8051eb851eb85p+5);
    r[8 * KQ_S] = kq_kmtf(c, 0x1.374bc6a7ef9dbp-6, 0x1.56415534e5baep-17, 0x1.3033333333333p+6);
    r[9 * KQ_S] = kq_kmtf(c, 0x1.da5119ce075f7p-4, 0x1.3d16e1c3d4d68p-16, 0x1.23b020c49ba5ep+5);
    r[10 * KQ_S] = kq_kmtf(c, 0x1.78d4fdf3b645ap-6, 0x1.81e03f705857bp-17, 0x1.d051eb851eb85p+5);
    r[11 * KQ_S] = kq_kmtf(c, 0x1.78d4fdf3b645ap-6, 0x1.81e03f705857bp-17, 0x1.203d70a3d70a4p+6);
    r[12 * KQ_S] = kq_kmtf(c, 0x1.47ae147ae147bp-7, 0x1.5cf751db94e6bp-17, 0x1.08147ae147ae1p+5);
    r[13 * KQ_S] = kq_kmtf(c, 0x1.89374bc6a7efap-10, 0x1.421f5f40d8376p-16, 0x1.70147ae147ae1p+5);
    r[14 * KQ_S] = kq_kmtf(c, 0x1.0000000000000p-1, 0x1.b43526527a205p-17, 0x1.78147ae147ae1p+5);
    r[15 * KQ_S] = kq_kmtf(c, 0x1.999999999999ap-4, 0x1.b43526527a205p-17, 0x1.3c0a3d70a3d71p+6);
    r[16 * KQ_S] = kq_kmtb(c, c.henry[0], 0x1.c28f5c28f5c29p-4, 0x1.ad7f29abcaf48p-17, 0x1.004189374bc6ap+6);
    r[17 * KQ_S] = kq_kmtb(c, c.henry[1], 0x1.63886594af4f1p-4, 0x1.baeb22f9294c3p-17, 0x1.f81a9fbe76c8bp+5);
    r[18 * KQ_S] = kq_kmtb(c, c.henry[2], 0x1.3a92a30553261p-13, 0x1.040bfe3b03e21p-16, 0x1.60147ae147ae1p+5);
    r[19 * KQ_S] = kq_kmtb(c, c.henry[3], 0x1.74bc6a7ef9db2p-4, 0x1.81e03f705857bp-16, 0x1.107ef9db22d0ep+4);
    r[20 * KQ_S] = kq_kmtb(c, c.henry[4], 0x1.39c0ebedfa440p-3, 0x1.e9e50b87f37efp-17, 0x1.101eb851eb852p+5);
    r[21 * KQ_S] = kq_kmtb(c, c.henry[5], 0x1.999999999999ap-4, 0x1.f09b082ea2aacp-17, 0x1.7ffbe76c8b439p+5);
    r[22 * KQ_S] = kq_kmtb(c, c.henry[6], 0x1.77318fc504817p-6, 0x1.00b0ffe7ac4c2p-16, 0x1.7033333333333p+5);
    r[23 * KQ_S] = kq_kmtb(c, c.henry[7], 0x1.bae46cfc829d0p-8, 0x1.b79024a5d1b64p-17, 0x1.8051eb851eb85p+5);
    r[24 * KQ_S] = kq_kmtb(c, c.henry[8], 0x1.374bc6a7ef9dbp-6, 0x1.56415534e5baep-17, 0x1.3033333333333p+6);
    r[25 * KQ_S] = kq_kmtb(c, c.henry[9], 0x1.da5119ce075f7p-4, 0x1.3d16e1c3d4d68p-16, 0x1.23b020c49ba5ep+5);
    r[26 * KQ_S] = kq_kmtb(c, c.henry[10], 0x1.78d4fdf3b645ap-6, 0x1.81e03f705857bp-17, 0x1.d051eb851eb85p+5);
    r[27 * KQ_S] = kq_kmtb(c, c.henry[11], 0x1.78d4fdf3b645ap-6, 0x1.81e03f705857bp-17, 0x1.203d70a3d70a4p+6);
    r[28 * KQ_S] = kq_kmtb(c, c.henry[12], 0x1.47ae147ae147bp-7, 0x1.5cf751db94e6bp-17, 0x1.08147ae147ae1p+5);
    r[29 * KQ_S] = kq_kmtb(c, c.henry[13], 0x1.89374bc6a7efap-10, 0x1.421f5f40d8376p-16, 0x1.70147ae147ae1p+5);
    r[30 * KQ_S] = kq_kmtb(c, c.henry[14], 0x1.0000000000000p-1, 0x1.b43526527a205p-17, 0x1.78147ae147ae1p+5);
    r[31 * KQ_S] = kq_kmtb(c, c.henry[15], 0x1.999999999999ap-4, 0x1.b43526527a205p-17, 0x1.3c0a3d70a3d71p+6);
    r[32 * KQ_S] = c.alfa3;
    r[33 * KQ_S] = c.alfa3;
    r[34 * KQ_S] = c.alfa3;
    r[35 * KQ_S] = c.alfa3;
    r[36 * KQ_S] = c.alfa3;
    r[37 * KQ_S] = c.alfa3;
    r[38 * KQ_S] = c.alfa3;
    r[39 * KQ_S] = c.alfa3;
    r[91 * KQ_S] = 0x1.199999999999ap+0;
    r[95 * KQ_S] = c.wetfac;
    r[96 * KQ_S] = c.wetfac;
    r[97 * KQ_S] = c.wetfac;
    r[98 * KQ_S] = c.wetfac;
    r[99 * KQ_S] = c.wetfac;
    r[100 * KQ_S] = c.wetfac;
    r[101 * KQ_S] = c.wetfac;
    r[102 * KQ_S] = c.wetfac;
    r[103 * KQ_S] = c.wetfac;
    r[104 * KQ_S] = c.wetfac;
    r[105 * KQ_S] = c.wetfac;
    r[106 * KQ_S] = c.wetfac;
    r[107 * KQ_S] = c.wetfac;
    r[108 * KQ_S] = c.wetfac;
    r[109 * KQ_S] = c.wetfac;
    r[110 * KQ_S] = c.wetfac;
    r[111 * KQ_S] = c.wetfac;
    r[112 * KQ_S] = c.wetfac;
    r[113 * KQ_S] = c.wetfac;
    r[114 * KQ_S] = c.wetfac;
    r[115 * KQ_S] = c.wetfac;
    r[116 * KQ_S] = c.wetfac;
    r[117 * KQ_S] = c.wetfac;
    r[118 * KQ_S] = c.wetfac;
    r[119 * KQ_S] = c.wetfac;
    r[120 * KQ_S] = c.wetfac;
    r[121 * KQ_S] = c.wetfac;
    r[122 * KQ_S] = c.wetfac;
    r[123 * KQ_S] = c.wetfac;
    r[124 * KQ_S] = c.wetfac;
    r[125 * KQ_S] = c.wetfac;
    r[126 * KQ_S] = c.wetfac;
    r[127 * KQ_S] = c.wetfac;
    r[128 * KQ_S] = c.wetfac;
    r[129 * KQ_S] = c.wetfac;
    r[130 * KQ_S] = c.wetfac;
    r[131 * KQ_S] = c.wetfac;
    r[132 * KQ_S] = c.wetfac;
    r[133 * KQ_S] = c.wetfac;
    r[134 * KQ_S] = c.wetfac;
    r[135 * KQ_S] = c.wetfac;
    r[136 * KQ_S] = c.wetfac;
    r[137 * KQ_S] = kq_kmtf(c, 0x1.999999999999ap-5, 0x1.00b0ffe7ac4c2p-16, 0x1.101cac083126fp+4);
    r[138 * KQ_S] = kq_kmtb(c, c.henry[16], 0x1.999999999999ap-5, 0x1.00b0ffe7ac4c2p-16, 0x1.101cac083126fp+4);
    r[139 * KQ_S] = c.wetfac;
    r[140 * KQ_S] = kq_kmtf(c, 0x1.47ae147ae147bp-6, 0x1.4f8b588e368f1p-17, 0x1.d8851eb851eb8p+6);
    r[141 * KQ_S] = kq_kmtf(c, 0x1.47ae147ae147bp-6, 0x1.4f8b588e368f1p-17, 0x1.9800000000000p+6);
    r[142 * KQ_S] = kq_kmtf(c, 0x1.47ae147ae147bp-6, 0x1.4f8b588e368f1p-17, 0x1.9800000000000p+6);
    r[143 * KQ_S] = kq_kmtb(c, c.henry[17], 0x1.47ae147ae147bp-6, 0x1.4f8b588e368f1p-17, 0x1.d8851eb851eb8p+6);
    r[144 * KQ_S] = kq_kmtb(c, c.henry[18], 0x1.47ae147ae147bp-6, 0x1.4f8b588e368f1p-17, 0x1.9800000000000p+6);
    r[145 * KQ_S] = kq_kmtb(c, c.henry[19], 0x1.47ae147ae147bp-6, 0x1.4f8b588e368f1p-17, 0x1.9800000000000p+6);
    r[157 * KQ_S] = c.wetfac;
    r[158 * KQ_S] = c.wetfac;
    r[159 * KQ_S] = c.wetfac;
    r[160 * KQ_S] = c.wetfac;
    r[161 * KQ_S] = c.wetfac;
    r[162 * KQ_S] = c.wetfac;
    r[163 * KQ_S] = c.wetfac;
    r[164 * KQ_S] = c.wetfac;
    r[165 * KQ_S] = c.wetfac;
    r[166 * KQ_S] = kq_kmtf(c, 0x1.78d4fdf3b645ap-6, 0x1.81e03f705857bp-17, 0x1.e06a7ef9db22dp+5);
    r[167 * KQ_S] = kq_kmtf(c, 0x1.07c84b5dcc63fp-5, 0x1.a013305e6c9cep-17, 0x1.e06a7ef9db22dp+5);
    r[168 * KQ_S] = kq_kmtf(c, 0x1.47ae147ae147bp-6, 0x1.132576b20e04ap-16, 0x1.e07ae147ae148p+4);
    r[169 * KQ_S] = kq_kmtf(c, 0x1.47ae147ae147bp-6, 0x1.132576b20e04ap-16, 0x1.e07ae147ae148p+4);
    r[170 * KQ_S] = (double)c.mtpyrac * kq_kmtf(c, 0x1.07c84b5dcc63fp-5, 0x1.a013305e6c9cep-17, 0x1.603d70a3d70a4p+6);
    r[171 * KQ_S] = kq_kmtb(c, c.henry[20], 0x1.78d4fdf3b645ap-6, 0x1.81e03f705857bp-17, 0x1.e06a7ef9db22dp+5);
    r[172 * KQ_S] = kq_kmtb(c, c.henry[21], 0x1.07c84b5dcc63fp-5, 0x1.a013305e6c9cep-17, 0x1.e06a7ef9db22dp+5);
    r[173 * KQ_S] = kq_kmtb(c, c.henry[22], 0x1.47ae147ae147bp-6, 0x1.132576b20e04ap-16, 0x1.e07ae147ae148p+4);
    r[174 * KQ_S] = kq_kmtb(c, c.henry[22], 0x1.47ae147ae147bp-6, 0x1.132576b20e04ap-16, 0x1.e07ae147ae148p+4);
    r[175 * KQ_S] = (double)c.mtpyrac * kq_kmtb(c, c.henry[23], 0x1.07c84b5dcc63fp-5, 0x1.a013305e6c9cep-17, 0x1.603d70a3d70a4p+6);
    r[188 * KQ_S] = kq_hydf(c, 0x1.70a3d70a3d70ap-3, 0x1.f7c0000000000p+11);
    r[189 * KQ_S] = 0x1.4e3bcd35a8588p-8;
    r[190 * KQ_S] = kq_hydf(c, 0x1.70a3d70a3d70ap-3, 0x1.f7c0000000000p+11);
    r[191 * KQ_S] = 0x1.4e3bcd35a8588p-8;
    r[192 * KQ_S] = kq_kphot(c, 0x1.34b365f379dfcp-18, c.jh2o2);
    r[211 * KQ_S] = c.wetfac;
    r[212 * KQ_S] = c.wetfac;
    r[213 * KQ_S] = c.wetfac;
    r[214 * KQ_S] = c.wetfac;
    r[215 * KQ_S] = c.wetfac;
    r[216 * KQ_S] = c.wetfac;
    r[217 * KQ_S] = c.wetfac;
    r[218 * KQ_S] = c.wetfac;
    r[219 * KQ_S] = c.wetfac;
    r[220 * KQ_S] = c.wetfac;
    r[221 * KQ_S] = c.wetfac;
    r[222 * KQ_S] = c.wetfac;
    r[223 * KQ_S] = c.wetfac;
    r[224 * KQ_S] = c.wetfac;
    r[225 * KQ_S] = c.wetfac;
    r[226 * KQ_S] = c.wetfac;
    r[227 * KQ_S] = kq_kmtf(c, 0x1.999999999999ap-5, 0x1.4f8b588e368f1p-17, 0x1.f000000000000p+5);
    r[228 * KQ_S] = kq_kmtf(c, 0x1.999999999999ap-5, 0x1.c4fc1df3300dep-17, 0x1.8800000000000p+5);
    r[229 * KQ_S] = kq_kmtb(c, c.henry[24], 0x1.999999999999ap-5, 0x1.4f8b588e368f1p-17, 0x1.f000000000000p+5);
    r[230 * KQ_S] = kq_kmtb(c, c.henry[25], 0x1.999999999999ap-5, 0x1.c4fc1df3300dep-17, 0x1.8800000000000p+5);
    r[231 * KQ_S] = kq_kphot(c, 0x1.2ca5d05ea7ab3p-21, -0x1.0000000000000p+0);
    r[260 * KQ_S] = c.wetfac;
    r[261 * KQ_S] = c.wetfac;
    r[262 * KQ_S] = c.wetfac;
    r[263 * KQ_S] = c.wetfac;
    r[264 * KQ_S] = c.wetfac;
    r[265 * KQ_S] = c.wetfac;
    r[266 * KQ_S] = c.wetfac;
    r[267 * KQ_S] = c.wetfac;
    r[268 * KQ_S] = c.wetfac;
}

KQ_HD KQ_NOINLINE void kq_rates_update(const Cell& c, const double* v, const double* f, double* r)
{
    r[40 * KQ_S] = kq_disf(c, 0x1.c779a6b50b0f2p-7, 0x1.d380000000000p+10, 0x1.7d78400000000p+27, 0);
    r[41 * KQ_S] = kq_disf(c, 0x1.209f2e6f59483p-24, 0x1.6300000000000p+8, 0x1.74876e8000000p+35, 1);
    r[42 * KQ_S] = kq_disf(c, 0x1.1000000000000p+4, 0x0.0p+0, 0x1.74876e8000000p+35, 0);
    r[43 * KQ_S] = kq_disf(c, 0x1.cdb57fff13c6ep-22, -0x1.f180000000000p+9, 0x1.f400000000000p+15, 0);
    r[44 * KQ_S] = kq_disf(c, 0x1.9ba83b3532653p-35, -0x1.be40000000000p+10, 0x1.74876e8000000p+35, 1);
    r[45 * KQ_S] = kq_disf(c, 0x1.28f4ebcfc7531p-16, -0x1.6300000000000p+9, 0x1.faa3b50000000p+34, 0);
    r[46 * KQ_S] = kq_disf(c, 0x1.797cc39ffd60fp-13, -0x1.4000000000000p+4, 0x1.74876e8000000p+35, 0);
    r[47 * KQ_S] = kq_disf(c, 0x1.a8ce000000000p+20, 0x1.aea0000000000p+12, 0x1.74876e8000000p+35, 0);
    r[48 * KQ_S] = kq_disf(c, 0x1.9f0d3ef0faf29p-53, -0x1.b2b0000000000p+12, 0x1.04c533c000000p+37, 0);
    r[49 * KQ_S] = kq_disf(c, 0x1.f400000000000p+9, 0x0.0p+0, 0x1.74876e8000000p+35, 0);
    r[50 * KQ_S] = kq_disf(c, 0x1.4e3bcd35a8588p-7, 0x1.31a0000000000p+11, 0x1.74876e8000000p+36, 1);
    r[51 * KQ_S] = kq_disf(c, 0x1.0c6f7a0b5ed8dp-16, 0x0.0p+0, 0x1.74876e8000000p+35, 0);
    r[52 * KQ_S] = kq_disf(c, 0x1.15df6555c52e7p-11, -0x1.b800000000000p+10, 0x1.74876e8000000p+35, 0);
    r[53 * KQ_S] = kq_disf(c, 0x1.4f8b588e368f1p-17, 0x0.0p+0, 0x1.74876e8000000p+35, 0);
    r[54 * KQ_S] = kq_disb(c, 0x1.7d78400000000p+27, 2);
    r[55 * KQ_S] = kq_disb(c, 0x1.74876e8000000p+35, 1);
    r[56 * KQ_S] = kq_disb(c, 0x1.74876e8000000p+35, 2);
    r[57 * KQ_S] = kq_disb(c, 0x1.f400000000000p+15, 2);
    r[58 * KQ_S] = kq_disb(c, 0x1.74876e8000000p+35, 1);
    r[59 * KQ_S] = kq_disb(c, 0x1.faa3b50000000p+34, 2);
    r[60 * KQ_S] = kq_disb(c, 0x1.74876e8000000p+35, 2);
    r[61 * KQ_S] = kq_disb(c, 0x1.74876e8000000p+35, 2);
    r[62 * KQ_S] = kq_disb(c, 0x1.04c533c000000p+37, 2);
    r[63 * KQ_S] = kq_disb(c, 0x1.74876e8000000p+35, 2);
    r[64 * KQ_S] = kq_disb(c, 0x1.74876e8000000p+36, 1);
    r[65 * KQ_S] = kq_disb(c, 0x1.74876e8000000p+35, 2);
    r[66 * KQ_S] = kq_disb(c, 0x1.74876e8000000p+35, 2);
    r[67 * KQ_S] = kq_disb(c, 0x1.74876e8000000p+35, 2);
    r[68 * KQ_S] = kq_krxn(c, v, 0x1.1c31e80000000p+26, -0x1.294147ae147aep+12, 1, 0, 0);
    r[69 * KQ_S] = kq_krxn(c, v, 0x1.7700000000000p+14, 0x0.0p+0, 0, 1, 0);
    r[70 * KQ_S] = kq_krxn(c, v, 0x1.6954000000000p+18, -0x1.59ae147ae147bp+12, 0, 2, 0);
    r[71 * KQ_S] = kq_krxn(c, v, 0x1.65a0bc0000000p+30, -0x1.4a08f5c28f5c3p+12, 0, 3, 0);
    r[72 * KQ_S] = kq_krxn(c, v, 0x1.7700000000000p+9, 0x0.0p+0, 0, 0, 1);
    r[73 * KQ_S] = kq_krxn(c, v, 0x1.7700000000000p+9, 0x0.0p+0, 0, 0, 1);
    r[74 * KQ_S] = kq_krxn(c, v, 0x1.7700000000000p+9, 0x0.0p+0, 0, 0, 1);
    r[75 * KQ_S] = kq_krxn(c, v, 0x1.4500000000000p+11, 0x0.0p+0, 0, 0, 1);
    r[76 * KQ_S] = kq_krxn(c, v, 0x1.4500000000000p+11, 0x0.0p+0, 0, 0, 1);
    r[77 * KQ_S] = kq_krxn(c, v, 0x1.4500000000000p+11, 0x0.0p+0, 0, 0, 1);
    r[78 * KQ_S] = kq_krxn(c, v, 0x1.2a05f20000000p+33, 0x0.0p+0, 3, 0, 1);
    r[79 * KQ_S] = kq_krxn(c, v, 0x1.2a05f20000000p+33, 0x0.0p+0, 3, 0, 1);
    r[80 * KQ_S] = kq_krxn(c, v, 0x1.2a05f20000000p+33, 0x0.0p+0, 3, 0, 1);
    r[81 * KQ_S] = kq_krxn(c, v, 0x1.21eac00000000p+24, -0x1.daf0000000000p+11, 3, 0, 0);
    r[82 * KQ_S] = kq_krxn(c, v, 0x1.12a8800000000p+25, -0x1.f3e6666666666p+11, 3, 0, 0);
    r[83 * KQ_S] = kq_krxn(c, v, 0x1.5e00000000000p+9, 0x0.0p+0, 0, 0, 0);
    r[84 * KQ_S] = kq_krxn(c, v, 0x1.9546000000000p+19, -0x1.5180000000000p+11, 0, 0, 0);
    r[85 * KQ_S] = kq_krxn(c, v, 0x1.6e36000000000p+26, -0x1.c700000000000p+9, 0, 0, 0);
    r[86 * KQ_S] = kq_krxn(c, v, 0x1.65a0bc0000000p+30, -0x1.7700000000000p+10, 0, 0, 0);
    r[87 * KQ_S] = kq_krxn(c, v, 0x1.e848000000000p+20, 0x0.0p+0, 0, 0, 0);
    r[88 * KQ_S] = kq_krxn(c, v, 0x1.e848000000000p+20, 0x0.0p+0, 0, 0, 0);
    r[89 * KQ_S] = kq_krxn(c, v, 0x1.e848000000000p+20, 0x0.0p+0, 0, 0, 0);
    r[90 * KQ_S] = kq_krxn(c, v, 0x1.4244000000000p+18, 0x0.0p+0, 0, 0, 0);
    r[92 * KQ_S] = kq_krxn(c, v, 0x1.e848000000000p+18, -0x1.b580000000000p+12, 0, 0, 0);
    r[93 * KQ_S] = kq_krxn(c, v, 0x1.2a05f20000000p+33, 0x0.0p+0, 0, 0, 0);
    r[94 * KQ_S] = kq_krxn(c, v, 0x1.2a05f20000000p+33, 0x0.0p+0, 0, 0, 0);
    r[146 * KQ_S] = kq_kiepox(c, v, f, 0x1.d7dbf487fcb92p-11, 0x1.b79024a5d1b64p-17, 1);
    r[147 * KQ_S] = kq_kiepox(c, v, f, 0x1.2157689ca18bdp-7, 0x1.87ea6f9ff5ff2p-19, 1);
    r[148 * KQ_S] = kq_kiepox(c, v, f, 0x1.a36e2eb1c432dp-13, 0x1.87ea6f9ff5ff2p-19, 1);
    r[149 * KQ_S] = kq_kiepox(c, v, f, 0x1.a36e2eb1c432dp-13, 0x1.87ea6f9ff5ff2p-19, 1);
    r[150 * KQ_S] = kq_kiepox(c, v, f, 0x1.d7dbf487fcb92p-11, 0x1.b79024a5d1b64p-17, 0);
    r[151 * KQ_S] = kq_kiepox(c, v, f, 0x1.2157689ca18bdp-7, 0x1.87ea6f9ff5ff2p-19, 0);
    r[152 * KQ_S] = kq_kiepox(c, v, f, 0x1.a36e2eb1c432dp-13, 0x1.87ea6f9ff5ff2p-19, 0);
    r[153 * KQ_S] = kq_kiepox(c, v, f, 0x1.d7dbf487fcb92p-11, 0x1.b79024a5d1b64p-17, 2);
    r[154 * KQ_S] = kq_kiepox(c, v, f, 0x1.a36e2eb1c432dp-13, 0x1.87ea6f9ff5ff2p-19, 2);
    r[155 * KQ_S] = kq_kiepox(c, v, f, 0x1.d7dbf487fcb92p-11, 0x1.b79024a5d1b64p-17, 2);
    r[156 * KQ_S] = kq_kiepox(c, v, f, 0x1.a36e2eb1c432dp-13, 0x1.87ea6f9ff5ff2p-19, 2);
    r[176 * KQ_S] = kq_disf(c, 0x1.6bdb1a6d698fep-12, -0x1.0b00000000000p+8, 0x1.2a05f20000000p+34, 0);
    r[177 * KQ_S] = kq_disf(c, 0x1.cac083126e979p-5, -0x1.c500000000000p+8, 0x1.74876e8000000p+35, 0);
    r[178 * KQ_S] = kq_disf(c, 0x1.c6a99d1cdbd8ep-15, -0x1.9280000000000p+9, 0x1.74876e8000000p+35, 1);
    r[179 * KQ_S] = kq_disf(c, 0x1.a36e2eb1c432dp-9, 0x0.0p+0, 0x1.2a05f20000000p+34, 0);
    r[180 * KQ_S] = kq_disf(c, 0x1.3660e51d25aabp-13, -0x1.4200000000000p+6, 0x1.2a05f20000000p+34, 0);
    r[181 * KQ_S] = kq_disf(c, 0x1.2599ed7c6fbd2p-16, 0x1.7000000000000p+5, 0x1.74876e8000000p+35, 0);
    r[182 * KQ_S] = kq_disb(c, 0x1.2a05f20000000p+34, 2);
    r[183 * KQ_S] = kq_disb(c, 0x1.74876e8000000p+35, 2);
    r[184 * KQ_S] = kq_disb(c, 0x1.74876e8000000p+35, 1);
    r[185 * KQ_S] = kq_disb(c, 0x1.2a05f20000000p+34, 2);
    r[186 * KQ_S] = kq_disb(c, 0x1.2a05f20000000p+34, 2);
    r[187 * KQ_S] = kq_disb(c, 0x1.74876e8000000p+35, 2);
    r[193 * KQ_S] = kq_krxn(c, v, 0x1.dcd6500000000p+28, 0x0.0p+0, 0, 0, 0);
    r[194 * KQ_S] = kq_krxn(c, v, 0x1.dcd6500000000p+29, 0x0.0p+0, 0, 0, 0);
    r[195 * KQ_S] = kq_krxn(c, v, 0x1.1e1a300000000p+29, 0x0.0p+0, 0, 0, 0);
    r[196 * KQ_S] = kq_krxn(c, v, 0x1.9a14780000000p+29, 0x0.0p+0, 0, 0, 0);
    r[197 * KQ_S] = kq_krxn(c, v, 0x1.0642ac0000000p+30, -0x1.7b00000000000p+10, 0, 0, 0);
    r[198 * KQ_S] = kq_krxn(c, v, 0x1.1e1a300000000p+27, 0x0.0p+0, 0, 0, 0);
    r[199 * KQ_S] = kq_krxn(c, v, 0x1.1e1a300000000p+30, 0x0.0p+0, 0, 0, 0);
    r[200 * KQ_S] = kq_krxn(c, v, 0x1.55cc000000000p+20, 0x0.0p+0, 0, 0, 0);
    r[201 * KQ_S] = kq_krxn(c, v, 0x1.6694e00000000p+25, 0x0.0p+0, 0, 0, 0);
    r[202 * KQ_S] = kq_krxn(c, v, 0x1.d5f8800000000p+22, 0x0.0p+0, 0, 0, 0);
    r[203 * KQ_S] = kq_krxn(c, v, 0x1.4dc9380000000p+29, 0x0.0p+0, 0, 0, 0);
    r[204 * KQ_S] = kq_krxn(c, v, 0x1.c9c3800000000p+25, 0x0.0p+0, 0, 0, 0);
    r[205 * KQ_S] = kq_krxn(c, v, 0x1.c9c3800000000p+25, 0x0.0p+0, 0, 0, 0);
    r[206 * KQ_S] = kq_krxn(c, v, 0x1.e848000000000p+23, 0x0.0p+0, 0, 0, 0);
    r[207 * KQ_S] = kq_krxn(c, v, 0x1.443fd00000000p+26, 0x0.0p+0, 0, 0, 0);
    r[208 * KQ_S] = kq_krxn(c, v, 0x1.0642ac0000000p+30, -0x1.fe00000000000p+9, 0, 0, 0);
    r[209 * KQ_S] = kq_krxn(c, v, 0x1.c9c3800000000p+26, -0x1.ef00000000000p+9, 0, 0, 0);
    r[210 * KQ_S] = kq_krxn(c, v, 0x1.0642ac0000000p+30, -0x1.fe00000000000p+9, 0, 0, 0);
    r[232 * KQ_S] = kq_krxn(c, v, 0x1.ad27480000000p+31, -0x1.d100000000000p+9, 0, 0, 0);
    r[233 * KQ_S] = kq_krxn(c, v, 0x1.a13b860000000p+34, 0x0.0p+0, 0, 0, 0);
    r[234 * KQ_S] = kq_krxn(c, v, 0x1.04c533c000000p+35, -0x1.6800000000000p+9, 0, 0, 0);
    r[235 * KQ_S] = kq_krxn(c, v, 0x1.e848000000000p+24, -0x1.a900000000000p+10, 0, 0, 0);
    r[236 * KQ_S] = kq_krxn(c, v, 0x1.41dd760000000p+31, 0x0.0p+0, 0, 0, 0);
    r[237 * KQ_S] = kq_krxn(c, v, 0x1.ad27480000000p+30, 0x0.0p+0, 0, 0, 0);
    r[238 * KQ_S] = kq_krxn(c, v, 0x1.0c388d0000000p+32, 0x0.0p+0, 0, 0, 0);
    r[239 * KQ_S] = kq_krxn(c, v, 0x1.a9fbe76c8b439p-6, 0x0.0p+0, 4, 0, 0);
    r[240 * KQ_S] = kq_krxn(c, v, 0x1.86a0000000000p+16, 0x0.0p+0, 0, 0, 0);
    r[241 * KQ_S] = kq_krxn(c, v, 0x1.35f1b40000000p+30, -0x1.1300000000000p+11, 0, 0, 0);
    r[242 * KQ_S] = kq_krxn(c, v, 0x1.0642ac0000000p+30, 0x0.0p+0, 0, 0, 0);
    r[243 * KQ_S] = kq_krxn(c, v, 0x1.954fc40000000p+30, 0x0.0p+0, 0, 0, 0);
    r[244 * KQ_S] = kq_krxn(c, v, 0x1.a39de00000000p+27, -0x1.4500000000000p+11, 0, 0, 0);
    r[245 * KQ_S] = kq_krxn(c, v, 0x1.b159800000000p+22, 0x0.0p+0, 3, 0, 0);
    r[246 * KQ_S] = kq_krxn(c, v, 0x1.cc00000000000p+8, -0x1.1300000000000p+10, 0, 0, 0);
    r[247 * KQ_S] = kq_krxn(c, v, 0x1.443fd00000000p+27, -0x1.1300000000000p+11, 0, 0, 0);
    r[248 * KQ_S] = kq_krxn(c, v, 0x1.e848000000000p+18, 0x0.0p+0, 0, 0, 0);
    r[249 * KQ_S] = kq_krxn(c, v, 0x1.954fc40000000p+31, -0x1.2c00000000000p+10, 0, 0, 0);
    r[250 * KQ_S] = kq_krxn(c, v, 0x1.8b00000000000p+9, -0x1.6a80000000000p+11, 0, 0, 0);
    r[251 * KQ_S] = kq_krxn(c, v, 0x1.7d78400000000p+24, -0x1.3240000000000p+11, 0, 0, 0);
    r[252 * KQ_S] = kq_krxn(c, v, 0x1.f8a0902de00d2p-8, -0x1.1f80000000000p+13, 4, 0, 0);
    r[253 * KQ_S] = kq_krxn(c, v, 0x1.ce80000000000p+11, 0x0.0p+0, 0, 0, 0);
    r[254 * KQ_S] = kq_krxn(c, v, 0x1.1e1a300000000p+28, 0x0.0p+0, 0, 0, 0);
    r[255 * KQ_S] = kq_krxn(c, v, 0x1.8b00000000000p+9, -0x1.6a80000000000p+11, 0, 0, 0);
    r[256 * KQ_S] = kq_krxn(c, v, 0x1.7d78400000000p+24, -0x1.3240000000000p+11, 0, 0, 0);
    r[257 * KQ_S] = kq_krxn(c, v, 0x1.f8a0902de00d2p-8, -0x1.1f80000000000p+13, 4, 0, 0);
    r[258 * KQ_S] = kq_krxn(c, v, 0x1.ce80000000000p+11, 0x0.0p+0, 0, 0, 0);
    r[259 * KQ_S] = kq_krxn(c, v, 0x1.1e1a300000000p+28, 0x0.0p+0, 0, 0, 0);
}

KQ_HD inline double kq_rtol(int i) { return (i == 101 || i == 105 || i == 112 || i == 145) ? 0x1.0624dd2f1a9fcp-10 : 0x1.47ae147ae147bp-7; }
KQ_HD inline double kq_atol(int) { return 0x1.47ae147ae147bp-7; }

KQ_HD inline void kq_add_diagonal(double* g, double x)
{
    g[0 * KQ_S] = g[0 * KQ_S] + x;
    g[1 * KQ_S] = g[1 * KQ_S] + x;
    g[2 * KQ_S] = g[2 * KQ_S] + x;
    g[3 * KQ_S] = g[3 * KQ_S] + x;
    g[4 * KQ_S] = g[4 * KQ_S] + x;
    g[5 * KQ_S] = g[5 * KQ_S] + x;
    g[6 * KQ_S] = g[6 * KQ_S] + x;
    g[7 * KQ_S] = g[7 * KQ_S] + x;
    g[9 * KQ_S] = g[9 * KQ_S] + x;
    g[11 * KQ_S] = g[11 * KQ_S] + x;
    g[12 * KQ_S] = g[12 * KQ_S] + x;
    g[14 * KQ_S] = g[14 * KQ_S] + x;
    g[15 * KQ_S] = g[15 * KQ_S] + x;
    g[16 * KQ_S] = g[16 * KQ_S] + x;
    g[17 * KQ_S] = g[17 * KQ_S] + x;
    g[18 * KQ_S] = g[18 * KQ_S] + x;
    g[19 * KQ_S] = g[19 * KQ_S] + x;
    g[21 * KQ_S] = g[21 * KQ_S] + x;
    g[22 * KQ_S] = g[22 * KQ_S] + x;
    g[31 * KQ_S] = g[31 * KQ_S] + x;
    g[33 * KQ_S] = g[33 * KQ_S] + x;
    g[38 * KQ_S] = g[38 * KQ_S] + x;
    g[42 * KQ_S] = g[42 * KQ_S] + x;
    g[44 * KQ_S] = g[44 * KQ_S] + x;
    g[46 * KQ_S] = g[46 * KQ_S] + x;
    g[48 * KQ_S] = g[48 * KQ_S] + x;
    g[51 * KQ_S] = g[51 * KQ_S] + x;
    g[53 * KQ_S] = g[53 * KQ_S] + x;
    g[55 * KQ_S] = g[55 * KQ_S] + x;
    g[59 * KQ_S] = g[59 * KQ_S] + x;
    g[61 * KQ_S] = g[61 * KQ_S] + x;
    g[63 * KQ_S] = g[63 * KQ_S] + x;
    g[65 * KQ_S] = g[65 * KQ_S] + x;
    g[67 * KQ_S] = g[67 * KQ_S] + x;
    g[69 * KQ_S] = g[69 * KQ_S] + x;
    g[71 * KQ_S] = g[71 * KQ_S] + x;
    g[74 * KQ_S] = g[74 * KQ_S] + x;
    g[76 * KQ_S] = g[76 * KQ_S] + x;
    g[78 * KQ_S] = g[78 * KQ_S] + x;
    g[80 * KQ_S] = g[80 * KQ_S] + x;
    g[82 * KQ_S] = g[82 * KQ_S] + x;
    g[84 * KQ_S] = g[84 * KQ_S] + x;
    g[85 * KQ_S] = g[85 * KQ_S] + x;
    g[88 * KQ_S] = g[88 * KQ_S] + x;
    g[90 * KQ_S] = g[90 * KQ_S] + x;
    g[92 * KQ_S] = g[92 * KQ_S] + x;
    g[94 * KQ_S] = g[94 * KQ_S] + x;
    g[95 * KQ_S] = g[95 * KQ_S] + x;
    g[97 * KQ_S] = g[97 * KQ_S] + x;
    g[100 * KQ_S] = g[100 * KQ_S] + x;
    g[103 * KQ_S] = g[103 * KQ_S] + x;
    g[105 * KQ_S] = g[105 * KQ_S] + x;
    g[108 * KQ_S] = g[108 * KQ_S] + x;
    g[112 * KQ_S] = g[112 * KQ_S] + x;
    g[114 * KQ_S] = g[114 * KQ_S] + x;
    g[116 * KQ_S] = g[116 * KQ_S] + x;
    g[120 * KQ_S] = g[120 * KQ_S] + x;
    g[122 * KQ_S] = g[122 * KQ_S] + x;
    g[124 * KQ_S] = g[124 * KQ_S] + x;
    g[126 * KQ_S] = g[126 * KQ_S] + x;
    g[129 * KQ_S] = g[129 * KQ_S] + x;
    g[131 * KQ_S] = g[131 * KQ_S] + x;
    g[135 * KQ_S] = g[135 * KQ_S] + x;
    g[138 * KQ_S] = g[138 * KQ_S] + x;
    g[142 * KQ_S] = g[142 * KQ_S] + x;
    g[145 * KQ_S] = g[145 * KQ_S] + x;
    g[148 * KQ_S] = g[148 * KQ_S] + x;
    g[152 * KQ_S] = g[152 * KQ_S] + x;
    g[155 * KQ_S] = g[155 * KQ_S] + x;
    g[157 * KQ_S] = g[157 * KQ_S] + x;
    g[160 * KQ_S] = g[160 * KQ_S] + x;
    g[164 * KQ_S] = g[164 * KQ_S] + x;
    g[166 * KQ_S] = g[166 * KQ_S] + x;
    g[168 * KQ_S] = g[168 * KQ_S] + x;
    g[170 * KQ_S] = g[170 * KQ_S] + x;
    g[173 * KQ_S] = g[173 * KQ_S] + x;
    g[175 * KQ_S] = g[175 * KQ_S] + x;
    g[178 * KQ_S] = g[178 * KQ_S] + x;
    g[180 * KQ_S] = g[180 * KQ_S] + x;
    g[182 * KQ_S] = g[182 * KQ_S] + x;
    g[184 * KQ_S] = g[184 * KQ_S] + x;
    g[186 * KQ_S] = g[186 * KQ_S] + x;
    g[188 * KQ_S] = g[188 * KQ_S] + x;
    g[190 * KQ_S] = g[190 * KQ_S] + x;
    g[192 * KQ_S] = g[192 * KQ_S] + x;
    g[194 * KQ_S] = g[194 * KQ_S] + x;
    g[196 * KQ_S] = g[196 * KQ_S] + x;
    g[198 * KQ_S] = g[198 * KQ_S] + x;
    g[200 * KQ_S] = g[200 * KQ_S] + x;
    g[202 * KQ_S] = g[202 * KQ_S] + x;
    g[204 * KQ_S] = g[204 * KQ_S] + x;
    g[206 * KQ_S] = g[206 * KQ_S] + x;
    g[208 * KQ_S] = g[208 * KQ_S] + x;
    g[210 * KQ_S] = g[210 * KQ_S] + x;
    g[212 * KQ_S] = g[212 * KQ_S] + x;
    g[214 * KQ_S] = g[214 * KQ_S] + x;
    g[216 * KQ_S] = g[216 * KQ_S] + x;
    g[218 * KQ_S] = g[218 * KQ_S] + x;
    g[220 * KQ_S] = g[220 * KQ_S] + x;
    g[222 * KQ_S] = g[222 * KQ_S] + x;
    g[224 * KQ_S] = g[224 * KQ_S] + x;
    g[226 * KQ_S] = g[226 * KQ_S] + x;
    g[228 * KQ_S] = g[228 * KQ_S] + x;
    g[231 * KQ_S] = g[231 * KQ_S] + x;
    g[237 * KQ_S] = g[237 * KQ_S] + x;
    g[241 * KQ_S] = g[241 * KQ_S] + x;
    g[244 * KQ_S] = g[244 * KQ_S] + x;
    g[248 * KQ_S] = g[248 * KQ_S] + x;
    g[253 * KQ_S] = g[253 * KQ_S] + x;
    g[255 * KQ_S] = g[255 * KQ_S] + x;
    g[259 * KQ_S] = g[259 * KQ_S] + x;
    g[264 * KQ_S] = g[264 * KQ_S] + x;
    g[267 * KQ_S] = g[267 * KQ_S] + x;
    g[269 * KQ_S] = g[269 * KQ_S] + x;
    g[273 * KQ_S] = g[273 * KQ_S] + x;
    g[279 * KQ_S] = g[279 * KQ_S] + x;
    g[282 * KQ_S] = g[282 * KQ_S] + x;
    g[287 * KQ_S] = g[287 * KQ_S] + x;
    g[296 * KQ_S] = g[296 * KQ_S] + x;
    g[302 * KQ_S] = g[302 * KQ_S] + x;
    g[306 * KQ_S] = g[306 * KQ_S] + x;
    g[310 * KQ_S] = g[310 * KQ_S] + x;
    g[313 * KQ_S] = g[313 * KQ_S] + x;
    g[319 * KQ_S] = g[319 * KQ_S] + x;
    g[326 * KQ_S] = g[326 * KQ_S] + x;
    g[337 * KQ_S] = g[337 * KQ_S] + x;
    g[342 * KQ_S] = g[342 * KQ_S] + x;
    g[345 * KQ_S] = g[345 * KQ_S] + x;
    g[350 * KQ_S] = g[350 * KQ_S] + x;
    g[355 * KQ_S] = g[355 * KQ_S] + x;
    g[360 * KQ_S] = g[360 * KQ_S] + x;
    g[366 * KQ_S] = g[366 * KQ_S] + x;
    g[372 * KQ_S] = g[372 * KQ_S] + x;
    g[378 * KQ_S] = g[378 * KQ_S] + x;
    g[383 * KQ_S] = g[383 * KQ_S] + x;
    g[390 * KQ_S] = g[390 * KQ_S] + x;
    g[396 * KQ_S] = g[396 * KQ_S] + x;
    g[400 * KQ_S] = g[400 * KQ_S] + x;
    g[405 * KQ_S] = g[405 * KQ_S] + x;
    g[410 * KQ_S] = g[410 * KQ_S] + x;
    g[418 * KQ_S] = g[418 * KQ_S] + x;
    g[423 * KQ_S] = g[423 * KQ_S] + x;
    g[431 * KQ_S] = g[431 * KQ_S] + x;
    g[438 * KQ_S] = g[438 * KQ_S] + x;
    g[446 * KQ_S] = g[446 * KQ_S] + x;
    g[452 * KQ_S] = g[452 * KQ_S] + x;
    g[462 * KQ_S] = g[462 * KQ_S] + x;
    g[470 * KQ_S] = g[470 * KQ_S] + x;
    g[480 * KQ_S] = g[480 * KQ_S] + x;
    g[488 * KQ_S] = g[488 * KQ_S] + x;
    g[494 * KQ_S] = g[494 * KQ_S] + x;
    g[505 * KQ_S] = g[505 * KQ_S] + x;
    g[528 * KQ_S] = g[528 * KQ_S] + x;
    g[555 * KQ_S] = g[555 * KQ_S] + x;
    g[584 * KQ_S] = g[584 * KQ_S] + x;
    g[632 * KQ_S] = g[632 * KQ_S] + x;
    g[657 * KQ_S] = g[657 * KQ_S] + x;
    g[669 * KQ_S] = g[669 * KQ_S] + x;
    g[685 * KQ_S] = g[685 * KQ_S] + x;
    g[700 * KQ_S] = g[700 * KQ_S] + x;
    g[737 * KQ_S] = g[737 * KQ_S] + x;
}

KQ_HD KQ_NOINLINE void kqu_fun_0(const double* v, const double* f, const double* r, double* vdot)
{
    vdot[0 * KQ_S] = 0.0 - (r[32 * KQ_S] * v[0 * KQ_S]);
    vdot[1 * KQ_S] = 0.0 - (r[33 * KQ_S] * v[1 * KQ_S]);
    vdot[2 * KQ_S] = 0.0 - (r[34 * KQ_S] * v[2 * KQ_S]);
    vdot[3 * KQ_S] = 0.0 - (r[35 * KQ_S] * v[3 * KQ_S]);
    vdot[4 * KQ_S] = 0.0 - (r[36 * KQ_S] * v[4 * KQ_S]);
    vdot[5 * KQ_S] = 0.0 - (r[37 * KQ_S] * v[5 * KQ_S]);
    vdot[6 * KQ_S] = 0.0 - (r[38 * KQ_S] * v[6 * KQ_S]);
    vdot[7 * KQ_S] = 0.0 - (r[39 * KQ_S] * v[7 * KQ_S]);
    vdot[8 * KQ_S] = 0.0 + (r[39 * KQ_S] * v[7 * KQ_S]) - (r[112 * KQ_S] * v[8 * KQ_S]);
    vdot[9 * KQ_S] = 0.0 + (r[37 * KQ_S] * v[5 * KQ_S]) - (r[113 * KQ_S] * v[9 * KQ_S]);
    vdot[10 * KQ_S] = 0.0 - (r[114 * KQ_S] * v[10 * KQ_S]);
    vdot[11 * KQ_S] = 0.0 + (r[38 * KQ_S] * v[6 * KQ_S]) - (r[115 * KQ_S] * v[11 * KQ_S]);
    vdot[12 * KQ_S] = 0.0 - (r[120 * KQ_S] * v[12 * KQ_S]);
    vdot[13 * KQ_S] = 0.0 - (r[121 * KQ_S] * v[13 * KQ_S]);
    vdot[14 * KQ_S] = 0.0 - (r[116 * KQ_S] * v[14 * KQ_S]);
    vdot[15 * KQ_S] = 0.0 - (r[117 * KQ_S] * v[15 * KQ_S]);
    vdot[16 * KQ_S] = 0.0 - (r[118 * KQ_S] * v[16 * KQ_S]);
    vdot[17 * KQ_S] = 0.0 + (r[35 * KQ_S] * v[3 * KQ_S]) - (r[119 * KQ_S] * v[17 * KQ_S]);
    vdot[18 * KQ_S] = 0.0 + (r[95 * KQ_S] * v[144 * KQ_S]) + (r[124 * KQ_S] * v[156 * KQ_S]) + (r[125 * KQ_S] * v[159 * KQ_S]) + (r[262 * KQ_S] * v[122 * KQ_S]) + (r[263 * KQ_S] * v[103 * KQ_S]) + (r[264 * KQ_S] * v[147 * KQ_S]) + (r[265 * KQ_S] * v[142 * KQ_S]) + (r[266 * KQ_S] * v[127 * KQ_S]);
    vdot[19 * KQ_S] = 0.0 + (r[96 * KQ_S] * v[106 * KQ_S]);
    vdot[20 * KQ_S] = 0.0 + (r[97 * KQ_S] * v[124 * KQ_S]) + (r[126 * KQ_S] * v[114 * KQ_S]) + (r[127 * KQ_S] * v[113 * KQ_S]) + (r[267 * KQ_S] * v[21 * KQ_S]);
    vdot[21 * KQ_S] = 0.0 + (r[201 * KQ_S] * v[131 * KQ_S] * v[160 * KQ_S]) + (r[202 * KQ_S] * v[130 * KQ_S] * v[160 * KQ_S]) - (r[267 * KQ_S] * v[21 * KQ_S]);
    vdot[22 * KQ_S] = 0.0 + (r[98 * KQ_S] * v[107 * KQ_S]);
    vdot[23 * KQ_S] = 0.0 + (r[99 * KQ_S] * v[145 * KQ_S]);
    vdot[24 * KQ_S] = 0.0 + (r[100 * KQ_S] * v[157 * KQ_S]);
    vdot[25 * KQ_S] = 0.0 + (r[101 * KQ_S] * v[141 * KQ_S]) + (r[128 * KQ_S] * v[137 * KQ_S]);
    vdot[26 * KQ_S] = 0.0 + (r[102 * KQ_S] * v[120 * KQ_S]);
    vdot[27 * KQ_S] = 0.0 + (r[103 * KQ_S] * v[121 * KQ_S]);
    vdot[28 * KQ_S] = 0.0 + (r[104 * KQ_S] * v[109 * KQ_S]) + (r[108 * KQ_S] * v[153 * KQ_S]) + (r[129 * KQ_S] * v[123 * KQ_S]);
    vdot[29 * KQ_S] = 0.0 + (r[105 * KQ_S] * v[110 * KQ_S]);
    vdot[30 * KQ_S] = 0.0 + (r[106 * KQ_S] * v[105 * KQ_S]);
    vdot[31 * KQ_S] = 0.0 + (r[107 * KQ_S] * v[112 * KQ_S]);
    vdot[32 * KQ_S] = 0.0 + (r[139 * KQ_S] * v[160 * KQ_S]);
    vdot[33 * KQ_S] = 0.0 + (r[109 * KQ_S] * v[146 * KQ_S]);
    vdot[34 * KQ_S] = 0.0 + (r[110 * KQ_S] * v[108 * KQ_S]);
    vdot[35 * KQ_S] = 0.0 + (r[111 * KQ_S] * v[111 * KQ_S]);
    vdot[36 * KQ_S] = 0.0 + (r[112 * KQ_S] * v[8 * KQ_S]);
    vdot[37 * KQ_S] = 0.0 + (r[120 * KQ_S] * v[12 * KQ_S]);
    vdot[38 * KQ_S] = 0.0 + (r[121 * KQ_S] * v[13 * KQ_S]);
    vdot[39 * KQ_S] = 0.0 + (r[113 * KQ_S] * v[9 * KQ_S]);
    vdot[40 * KQ_S] = 0.0 + (r[114 * KQ_S] * v[10 * KQ_S]);
    vdot[41 * KQ_S] = 0.0 + (r[115 * KQ_S] * v[11 * KQ_S]);
    vdot[42 * KQ_S] = 0.0 + (r[122 * KQ_S] * v[155 * KQ_S]);
    vdot[43 * KQ_S] = 0.0 + (r[116 * KQ_S] * v[14 * KQ_S]);
    vdot[44 * KQ_S] = 0.0 + (r[117 * KQ_S] * v[15 * KQ_S]);
    vdot[45 * KQ_S] = 0.0 + (r[118 * KQ_S] * v[16 * KQ_S]);
    vdot[46 * KQ_S] = 0.0 + (r[119 * KQ_S] * v[17 * KQ_S]);
    vdot[47 * KQ_S] = 0.0 + (r[132 * KQ_S] * v[158 * KQ_S]);
    vdot[48 * KQ_S] = 0.0 + (r[133 * KQ_S] * v[125 * KQ_S]) + (r[134 * KQ_S] * v[151 * KQ_S]);
    vdot[49 * KQ_S] = 0.0 + (r[135 * KQ_S] * v[129 * KQ_S]) + (r[136 * KQ_S] * v[149 * KQ_S]);
    vdot[50 * KQ_S] = 0.0 + (r[157 * KQ_S] * v[115 * KQ_S]);
    vdot[51 * KQ_S] = 0.0 + (r[158 * KQ_S] * v[101 * KQ_S]) + (r[165 * KQ_S] * v[52 * KQ_S]);
    vdot[52 * KQ_S] = 0.0 + (r[150 * KQ_S] * v[115 * KQ_S] * f[0 * KQ_S]) + (r[151 * KQ_S] * v[115 * KQ_S] * v[153 * KQ_S]) + (r[152 * KQ_S] * v[115 * KQ_S] * v[146 * KQ_S]) - (r[165 * KQ_S] * v[52 * KQ_S]);
    vdot[53 * KQ_S] = 0.0 + (r[159 * KQ_S] * v[102 * KQ_S]);
    vdot[54 * KQ_S] = 0.0 + (r[160 * KQ_S] * v[55 * KQ_S]);
    vdot[55 * KQ_S] = 0.0 + (r[148 * KQ_S] * v[101 * KQ_S] * v[115 * KQ_S]) + (r[149 * KQ_S] * v[102 * KQ_S] * v[115 * KQ_S]) - (r[160 * KQ_S] * v[55 * KQ_S]);
    vdot[56 * KQ_S] = 0.0 + (r[161 * KQ_S] * v[75 * KQ_S]);
    vdot[57 * KQ_S] = 0.0 + (r[162 * KQ_S] * v[77 * KQ_S]);
    vdot[58 * KQ_S] = 0.0 + (r[163 * KQ_S] * v[59 * KQ_S]);
    vdot[59 * KQ_S] = 0.0 + (r[153 * KQ_S] * v[75 * KQ_S] * f[0 * KQ_S]) + (r[155 * KQ_S] * v[77 * KQ_S] * f[0 * KQ_S]) - (r[163 * KQ_S] * v[59 * KQ_S]);
    vdot[60 * KQ_S] = 0.0 + (r[164 * KQ_S] * v[61 * KQ_S]);
    vdot[61 * KQ_S] = 0.0 + (r[154 * KQ_S] * v[75 * KQ_S] * v[153 * KQ_S]) + (r[156 * KQ_S] * v[77 * KQ_S] * v[153 * KQ_S]) - (r[164 * KQ_S] * v[61 * KQ_S]);
}

KQ_HD KQ_NOINLINE void kqu_fun_1(const double* v, const double* f, const double* r, double* vdot)
{
    vdot[62 * KQ_S] = 0.0 + (r[211 * KQ_S] * v[136 * KQ_S]) + (r[212 * KQ_S] * v[140 * KQ_S]);
    vdot[63 * KQ_S] = 0.0 + (r[213 * KQ_S] * v[128 * KQ_S]) + (r[214 * KQ_S] * v[131 * KQ_S]) + (r[215 * KQ_S] * v[130 * KQ_S]);
    vdot[64 * KQ_S] = 0.0 + (r[216 * KQ_S] * v[133 * KQ_S]) + (r[217 * KQ_S] * v[132 * KQ_S]);
    vdot[65 * KQ_S] = 0.0 + (r[218 * KQ_S] * v[134 * KQ_S]) + (r[219 * KQ_S] * v[135 * KQ_S]);
    vdot[66 * KQ_S] = 0.0 + (r[220 * KQ_S] * v[148 * KQ_S]) + (r[224 * KQ_S] * v[143 * KQ_S]) + (r[264 * KQ_S] * v[147 * KQ_S]);
    vdot[67 * KQ_S] = 0.0 + (r[130 * KQ_S] * v[150 * KQ_S]) + (r[131 * KQ_S] * v[154 * KQ_S]);
    vdot[68 * KQ_S] = 0.0 + (r[221 * KQ_S] * v[104 * KQ_S]);
    vdot[69 * KQ_S] = 0.0 + (r[222 * KQ_S] * v[138 * KQ_S]) + (r[223 * KQ_S] * v[139 * KQ_S]);
    vdot[70 * KQ_S] = 0.0 + (r[225 * KQ_S] * v[118 * KQ_S]) + (r[226 * KQ_S] * v[116 * KQ_S]) + (r[268 * KQ_S] * v[117 * KQ_S]);
    vdot[71 * KQ_S] = 0.0 + (r[260 * KQ_S] * v[126 * KQ_S]);
    vdot[72 * KQ_S] = 0.0 + (r[261 * KQ_S] * v[119 * KQ_S]);
    vdot[73 * KQ_S] = 0.0 - (r[14 * KQ_S] * v[73 * KQ_S]) + (r[30 * KQ_S] * v[125 * KQ_S]);
    vdot[74 * KQ_S] = 0.0 - (r[141 * KQ_S] * v[74 * KQ_S]) + (r[144 * KQ_S] * v[75 * KQ_S]);
    vdot[75 * KQ_S] = 0.0 + (r[141 * KQ_S] * v[74 * KQ_S]) - (r[144 * KQ_S] * v[75 * KQ_S]) - (r[153 * KQ_S] * v[75 * KQ_S] * f[0 * KQ_S]) - (r[154 * KQ_S] * v[75 * KQ_S] * v[153 * KQ_S]) - (r[161 * KQ_S] * v[75 * KQ_S]);
    vdot[76 * KQ_S] = 0.0 - (r[142 * KQ_S] * v[76 * KQ_S]) + (r[145 * KQ_S] * v[77 * KQ_S]);
    vdot[77 * KQ_S] = 0.0 + (r[142 * KQ_S] * v[76 * KQ_S]) - (r[145 * KQ_S] * v[77 * KQ_S]) - (r[155 * KQ_S] * v[77 * KQ_S] * f[0 * KQ_S]) - (r[156 * KQ_S] * v[77 * KQ_S] * v[153 * KQ_S]) - (r[162 * KQ_S] * v[77 * KQ_S]);
    vdot[78 * KQ_S] = 0.0 - (r[166 * KQ_S] * v[78 * KQ_S]) + (r[171 * KQ_S] * v[104 * KQ_S]);
    vdot[79 * KQ_S] = 0.0 - (r[167 * KQ_S] * v[79 * KQ_S]) + (r[172 * KQ_S] * v[134 * KQ_S]);
    vdot[80 * KQ_S] = 0.0 - (r[168 * KQ_S] * v[80 * KQ_S]) + (r[173 * KQ_S] * v[143 * KQ_S]);
    vdot[81 * KQ_S] = 0.0 - (r[12 * KQ_S] * v[81 * KQ_S]) + (r[28 * KQ_S] * v[154 * KQ_S]);
    vdot[82 * KQ_S] = 0.0 - (r[170 * KQ_S] * v[82 * KQ_S]) + (r[175 * KQ_S] * v[133 * KQ_S]);
    vdot[83 * KQ_S] = 0.0 - (r[169 * KQ_S] * v[83 * KQ_S]) + (r[174 * KQ_S] * v[118 * KQ_S]);
    vdot[84 * KQ_S] = 0.0 - (r[4 * KQ_S] * v[84 * KQ_S]) + (r[20 * KQ_S] * v[145 * KQ_S]);
    vdot[85 * KQ_S] = 0.0 - (r[1 * KQ_S] * v[85 * KQ_S]) + (r[17 * KQ_S] * v[106 * KQ_S]);
    vdot[86 * KQ_S] = 0.0 - (r[2 * KQ_S] * v[86 * KQ_S]) + (r[18 * KQ_S] * v[124 * KQ_S]);
    vdot[87 * KQ_S] = 0.0 - (r[3 * KQ_S] * v[87 * KQ_S]) + (r[19 * KQ_S] * v[107 * KQ_S]);
    vdot[88 * KQ_S] = 0.0 - (r[5 * KQ_S] * v[88 * KQ_S]) + (r[21 * KQ_S] * v[157 * KQ_S]);
    vdot[89 * KQ_S] = 0.0 - (r[6 * KQ_S] * v[89 * KQ_S]) + (r[22 * KQ_S] * v[141 * KQ_S]);
    vdot[90 * KQ_S] = 0.0 - (r[7 * KQ_S] * v[90 * KQ_S]) + (r[23 * KQ_S] * v[120 * KQ_S]);
    vdot[91 * KQ_S] = 0.0 - (r[8 * KQ_S] * v[91 * KQ_S]) + (r[24 * KQ_S] * v[121 * KQ_S]);
    vdot[92 * KQ_S] = 0.0 - (r[9 * KQ_S] * v[92 * KQ_S]) + (r[25 * KQ_S] * v[110 * KQ_S]);
    vdot[93 * KQ_S] = 0.0 - (r[10 * KQ_S] * v[93 * KQ_S]) + (r[26 * KQ_S] * v[105 * KQ_S]);
    vdot[94 * KQ_S] = 0.0 - (r[11 * KQ_S] * v[94 * KQ_S]) + (r[27 * KQ_S] * v[112 * KQ_S]);
    vdot[95 * KQ_S] = 0.0 - (r[13 * KQ_S] * v[95 * KQ_S]) + (r[29 * KQ_S] * v[158 * KQ_S]);
    vdot[96 * KQ_S] = 0.0 - (r[15 * KQ_S] * v[96 * KQ_S]) + (r[31 * KQ_S] * v[149 * KQ_S]);
    vdot[97 * KQ_S] = 0.0 - (r[227 * KQ_S] * v[97 * KQ_S]) + (r[229 * KQ_S] * v[126 * KQ_S]);
    vdot[98 * KQ_S] = 0.0 - (r[228 * KQ_S] * v[98 * KQ_S]) + (r[230 * KQ_S] * v[119 * KQ_S]);
    vdot[99 * KQ_S] = 0.0 - (r[0 * KQ_S] * v[99 * KQ_S]) + (r[16 * KQ_S] * v[144 * KQ_S]);
    vdot[100 * KQ_S] = 0.0 - (r[140 * KQ_S] * v[100 * KQ_S]) + (r[143 * KQ_S] * v[115 * KQ_S]);
    vdot[101 * KQ_S] = 0.0 + (r[146 * KQ_S] * v[115 * KQ_S] * f[0 * KQ_S]) - (r[148 * KQ_S] * v[101 * KQ_S] * v[115 * KQ_S]) - (r[158 * KQ_S] * v[101 * KQ_S]);
    vdot[102 * KQ_S] = 0.0 + (r[147 * KQ_S] * v[115 * KQ_S] * v[153 * KQ_S]) - (r[149 * KQ_S] * v[102 * KQ_S] * v[115 * KQ_S]) - (r[159 * KQ_S] * v[102 * KQ_S]);
}

KQ_HD KQ_NOINLINE void kqu_fun_2(const double* v, const double* f, const double* r, double* vdot)
{
    vdot[103 * KQ_S] = 0.0 + (r[236 * KQ_S] * v[156 * KQ_S] * v[160 * KQ_S]) + (r[241 * KQ_S] * v[126 * KQ_S] * v[156 * KQ_S]) - (r[242 * KQ_S] * v[103 * KQ_S] * f[2 * KQ_S]) + (r[248 * KQ_S] * v[119 * KQ_S] * v[156 * KQ_S]) - (r[263 * KQ_S] * v[103 * KQ_S]);
    vdot[104 * KQ_S] = 0.0 + (r[166 * KQ_S] * v[78 * KQ_S]) - (r[171 * KQ_S] * v[104 * KQ_S]) - (r[193 * KQ_S] * v[104 * KQ_S] * v[160 * KQ_S]) - (r[194 * KQ_S] * v[104 * KQ_S] * v[160 * KQ_S]) - (r[221 * KQ_S] * v[104 * KQ_S]);
    vdot[105 * KQ_S] = 0.0 + (r[10 * KQ_S] * v[93 * KQ_S]) - (r[26 * KQ_S] * v[105 * KQ_S]) - (r[106 * KQ_S] * v[105 * KQ_S]) + (r[194 * KQ_S] * v[104 * KQ_S] * v[160 * KQ_S]) - (r[197 * KQ_S] * v[105 * KQ_S] * v[160 * KQ_S]);
    vdot[106 * KQ_S] = 0.0 + (r[1 * KQ_S] * v[85 * KQ_S]) - (r[17 * KQ_S] * v[106 * KQ_S]) - (r[42 * KQ_S] * v[106 * KQ_S]) + (r[56 * KQ_S] * v[146 * KQ_S] * v[155 * KQ_S]) - (r[96 * KQ_S] * v[106 * KQ_S]);
    vdot[107 * KQ_S] = 0.0 + (r[3 * KQ_S] * v[87 * KQ_S]) - (r[19 * KQ_S] * v[107 * KQ_S]) - (r[45 * KQ_S] * v[107 * KQ_S]) + (r[59 * KQ_S] * v[108 * KQ_S] * v[152 * KQ_S]) - (r[98 * KQ_S] * v[107 * KQ_S]);
    vdot[108 * KQ_S] = 0.0 + (r[33 * KQ_S] * v[1 * KQ_S]) + (r[45 * KQ_S] * v[107 * KQ_S]) - (r[59 * KQ_S] * v[108 * KQ_S] * v[152 * KQ_S]) - (r[110 * KQ_S] * v[108 * KQ_S]);
    vdot[109 * KQ_S] = 0.0 - (r[49 * KQ_S] * v[109 * KQ_S]) + (r[63 * KQ_S] * v[123 * KQ_S] * v[155 * KQ_S]) - (r[104 * KQ_S] * v[109 * KQ_S]);
    vdot[110 * KQ_S] = 0.0 + (r[9 * KQ_S] * v[92 * KQ_S]) - (r[25 * KQ_S] * v[110 * KQ_S]) - (r[47 * KQ_S] * v[110 * KQ_S]) + (r[61 * KQ_S] * v[111 * KQ_S] * v[155 * KQ_S]) - (r[105 * KQ_S] * v[110 * KQ_S]);
    vdot[111 * KQ_S] = 0.0 + (r[34 * KQ_S] * v[2 * KQ_S]) + (r[47 * KQ_S] * v[110 * KQ_S]) - (r[61 * KQ_S] * v[111 * KQ_S] * v[155 * KQ_S]) - (r[111 * KQ_S] * v[111 * KQ_S]);
    vdot[112 * KQ_S] = 0.0 + (r[11 * KQ_S] * v[94 * KQ_S]) - (r[27 * KQ_S] * v[112 * KQ_S]) - (r[107 * KQ_S] * v[112 * KQ_S]) - (r[203 * KQ_S] * v[112 * KQ_S] * v[160 * KQ_S]);
    vdot[113 * KQ_S] = 0.0 + (r[44 * KQ_S] * v[114 * KQ_S]) - (r[58 * KQ_S] * v[113 * KQ_S] * v[155 * KQ_S]) - (r[127 * KQ_S] * v[113 * KQ_S]);
    vdot[114 * KQ_S] = 0.0 + (r[43 * KQ_S] * v[124 * KQ_S]) - (r[44 * KQ_S] * v[114 * KQ_S]) - (r[57 * KQ_S] * v[114 * KQ_S] * v[155 * KQ_S]) + (r[58 * KQ_S] * v[113 * KQ_S] * v[155 * KQ_S]) - (r[126 * KQ_S] * v[114 * KQ_S]);
    vdot[115 * KQ_S] = 0.0 + (r[140 * KQ_S] * v[100 * KQ_S]) - (r[143 * KQ_S] * v[115 * KQ_S]) - (r[146 * KQ_S] * v[115 * KQ_S] * f[0 * KQ_S]) - (r[147 * KQ_S] * v[115 * KQ_S] * v[153 * KQ_S]) - (r[148 * KQ_S] * v[101 * KQ_S] * v[115 * KQ_S]) - (r[149 * KQ_S] * v[102 * KQ_S] * v[115 * KQ_S]) - (r[150 * KQ_S] * v[115 * KQ_S] * f[0 * KQ_S]) - (r[151 * KQ_S] * v[115 * KQ_S] * v[153 * KQ_S]) - (r[152 * KQ_S] * v[115 * KQ_S] * v[146 * KQ_S]) - (r[157 * KQ_S] * v[115 * KQ_S]);
    vdot[116 * KQ_S] = 0.0 + (r[190 * KQ_S] * v[118 * KQ_S] * f[0 * KQ_S]) - (r[191 * KQ_S] * v[116 * KQ_S]) - (r[210 * KQ_S] * v[116 * KQ_S] * v[160 * KQ_S]) - (r[226 * KQ_S] * v[116 * KQ_S]) + (r[258 * KQ_S] * v[117 * KQ_S] * v[152 * KQ_S]);
    vdot[117 * KQ_S] = 0.0 + (r[255 * KQ_S] * v[118 * KQ_S] * v[156 * KQ_S]) + (r[256 * KQ_S] * v[118 * KQ_S] * v[159 * KQ_S]) - (r[257 * KQ_S] * v[117 * KQ_S]) - (r[258 * KQ_S] * v[117 * KQ_S] * v[152 * KQ_S]) - (r[259 * KQ_S] * v[117 * KQ_S] * v[160 * KQ_S]) - (r[268 * KQ_S] * v[117 * KQ_S]);
    vdot[118 * KQ_S] = 0.0 + (r[169 * KQ_S] * v[83 * KQ_S]) - (r[174 * KQ_S] * v[118 * KQ_S]) - (r[190 * KQ_S] * v[118 * KQ_S] * f[0 * KQ_S]) + (r[191 * KQ_S] * v[116 * KQ_S]) - (r[225 * KQ_S] * v[118 * KQ_S]) - (r[255 * KQ_S] * v[118 * KQ_S] * v[156 * KQ_S]) - (r[256 * KQ_S] * v[118 * KQ_S] * v[159 * KQ_S]) + (r[257 * KQ_S] * v[117 * KQ_S]);
}

KQ_HD KQ_NOINLINE void kqu_fun_3(const double* v, const double* f, const double* r, double* vdot)
{
    vdot[119 * KQ_S] = 0.0 + (r[228 * KQ_S] * v[98 * KQ_S]) - (r[230 * KQ_S] * v[119 * KQ_S]) + -0x1.0000000000000p+1 * (r[247 * KQ_S] * v[119 * KQ_S] * v[119 * KQ_S]) - (r[248 * KQ_S] * v[119 * KQ_S] * v[156 * KQ_S]) - (r[261 * KQ_S] * v[119 * KQ_S]);
    vdot[120 * KQ_S] = 0.0 + (r[7 * KQ_S] * v[90 * KQ_S]) - (r[23 * KQ_S] * v[120 * KQ_S]) - (r[81 * KQ_S] * v[120 * KQ_S] * v[155 * KQ_S] * v[156 * KQ_S]) - (r[102 * KQ_S] * v[120 * KQ_S]) + (r[248 * KQ_S] * v[119 * KQ_S] * v[156 * KQ_S]);
    vdot[121 * KQ_S] = 0.0 + (r[8 * KQ_S] * v[91 * KQ_S]) - (r[24 * KQ_S] * v[121 * KQ_S]) - (r[82 * KQ_S] * v[121 * KQ_S] * v[155 * KQ_S] * v[156 * KQ_S]) - (r[83 * KQ_S] * v[121 * KQ_S] * v[156 * KQ_S]) - (r[103 * KQ_S] * v[121 * KQ_S]);
    vdot[122 * KQ_S] = 0.0 + (r[240 * KQ_S] * v[126 * KQ_S] * v[153 * KQ_S]) + 0x1.0000000000000p+1 * (r[244 * KQ_S] * v[142 * KQ_S] * v[142 * KQ_S]) - (r[246 * KQ_S] * v[122 * KQ_S] * f[0 * KQ_S]) - (r[262 * KQ_S] * v[122 * KQ_S]);
    vdot[123 * KQ_S] = 0.0 + (r[49 * KQ_S] * v[109 * KQ_S]) - (r[50 * KQ_S] * v[123 * KQ_S]) - (r[63 * KQ_S] * v[123 * KQ_S] * v[155 * KQ_S]) + (r[64 * KQ_S] * v[153 * KQ_S] * v[155 * KQ_S]) - (r[129 * KQ_S] * v[123 * KQ_S]) + (r[246 * KQ_S] * v[122 * KQ_S] * f[0 * KQ_S]);
    vdot[124 * KQ_S] = 0.0 + (r[2 * KQ_S] * v[86 * KQ_S]) - (r[18 * KQ_S] * v[124 * KQ_S]) - (r[43 * KQ_S] * v[124 * KQ_S]) + (r[57 * KQ_S] * v[114 * KQ_S] * v[155 * KQ_S]) - (r[97 * KQ_S] * v[124 * KQ_S]) + 0x1.0000000000000p+1 * (r[200 * KQ_S] * v[128 * KQ_S] * v[160 * KQ_S]) + (r[201 * KQ_S] * v[131 * KQ_S] * v[160 * KQ_S]) + (r[202 * KQ_S] * v[130 * KQ_S] * v[160 * KQ_S]) + (r[204 * KQ_S] * v[133 * KQ_S] * v[160 * KQ_S]) + (r[205 * KQ_S] * v[132 * KQ_S] * v[160 * KQ_S]) + (r[209 * KQ_S] * v[141 * KQ_S] * v[160 * KQ_S]) + (r[249 * KQ_S] * v[137 * KQ_S] * v[160 * KQ_S]);
    vdot[125 * KQ_S] = 0.0 + (r[14 * KQ_S] * v[73 * KQ_S]) - (r[30 * KQ_S] * v[125 * KQ_S]) - (r[52 * KQ_S] * v[125 * KQ_S]) + (r[66 * KQ_S] * v[151 * KQ_S] * v[155 * KQ_S]) - (r[94 * KQ_S] * v[125 * KQ_S] * v[160 * KQ_S]) - (r[133 * KQ_S] * v[125 * KQ_S]);
    vdot[126 * KQ_S] = 0.0 + (r[227 * KQ_S] * v[97 * KQ_S]) - (r[229 * KQ_S] * v[126 * KQ_S]) - (r[240 * KQ_S] * v[126 * KQ_S] * v[153 * KQ_S]) - (r[241 * KQ_S] * v[126 * KQ_S] * v[156 * KQ_S]) - (r[260 * KQ_S] * v[126 * KQ_S]);
    vdot[127 * KQ_S] = 0.0 + (r[243 * KQ_S] * v[142 * KQ_S] * v[154 * KQ_S]) - (r[245 * KQ_S] * v[127 * KQ_S] * v[155 * KQ_S] * v[156 * KQ_S]) - (r[266 * KQ_S] * v[127 * KQ_S]);
    vdot[128 * KQ_S] = 0.0 - (r[177 * KQ_S] * v[128 * KQ_S]) + (r[183 * KQ_S] * v[131 * KQ_S] * v[155 * KQ_S]) + (r[198 * KQ_S] * v[136 * KQ_S] * v[160 * KQ_S]) - (r[200 * KQ_S] * v[128 * KQ_S] * v[160 * KQ_S]) - (r[213 * KQ_S] * v[128 * KQ_S]);
    vdot[129 * KQ_S] = 0.0 + (r[53 * KQ_S] * v[149 * KQ_S]) - (r[67 * KQ_S] * v[129 * KQ_S] * v[155 * KQ_S]) - (r[91 * KQ_S] * v[129 * KQ_S]) - (r[135 * KQ_S] * v[129 * KQ_S]) + (r[238 * KQ_S] * v[150 * KQ_S] * v[158 * KQ_S]);
    vdot[130 * KQ_S] = 0.0 + (r[178 * KQ_S] * v[131 * KQ_S]) - (r[184 * KQ_S] * v[130 * KQ_S] * v[155 * KQ_S]) - (r[202 * KQ_S] * v[130 * KQ_S] * v[160 * KQ_S]) - (r[215 * KQ_S] * v[130 * KQ_S]);
    vdot[131 * KQ_S] = 0.0 + (r[177 * KQ_S] * v[128 * KQ_S]) - (r[178 * KQ_S] * v[131 * KQ_S]) - (r[183 * KQ_S] * v[131 * KQ_S] * v[155 * KQ_S]) + (r[184 * KQ_S] * v[130 * KQ_S] * v[155 * KQ_S]) + (r[199 * KQ_S] * v[140 * KQ_S] * v[160 * KQ_S]) - (r[201 * KQ_S] * v[131 * KQ_S] * v[160 * KQ_S]) - (r[214 * KQ_S] * v[131 * KQ_S]);
    vdot[132 * KQ_S] = 0.0 + (r[179 * KQ_S] * v[133 * KQ_S]) - (r[185 * KQ_S] * v[132 * KQ_S] * v[155 * KQ_S]) + 0x1.d70a3e0000000p-1 * (r[203 * KQ_S] * v[112 * KQ_S] * v[160 * KQ_S]) - (r[205 * KQ_S] * v[132 * KQ_S] * v[160 * KQ_S]) - (r[217 * KQ_S] * v[132 * KQ_S]);
}

KQ_HD KQ_NOINLINE void kqu_fun_4(const double* v, const double* f, const double* r, double* vdot)
{
    vdot[133 * KQ_S] = 0.0 + (r[170 * KQ_S] * v[82 * KQ_S]) - (r[175 * KQ_S] * v[133 * KQ_S]) - (r[179 * KQ_S] * v[133 * KQ_S]) + (r[185 * KQ_S] * v[132 * KQ_S] * v[155 * KQ_S]) - (r[204 * KQ_S] * v[133 * KQ_S] * v[160 * KQ_S]) - (r[216 * KQ_S] * v[133 * KQ_S]);
    vdot[134 * KQ_S] = 0.0 + (r[167 * KQ_S] * v[79 * KQ_S]) - (r[172 * KQ_S] * v[134 * KQ_S]) - (r[181 * KQ_S] * v[134 * KQ_S]) + (r[187 * KQ_S] * v[135 * KQ_S] * v[155 * KQ_S]) + (r[204 * KQ_S] * v[133 * KQ_S] * v[160 * KQ_S]) - (r[206 * KQ_S] * v[134 * KQ_S] * v[160 * KQ_S]) - (r[218 * KQ_S] * v[134 * KQ_S]);
    vdot[135 * KQ_S] = 0.0 + (r[181 * KQ_S] * v[134 * KQ_S]) - (r[187 * KQ_S] * v[135 * KQ_S] * v[155 * KQ_S]) + (r[205 * KQ_S] * v[132 * KQ_S] * v[160 * KQ_S]) - (r[207 * KQ_S] * v[135 * KQ_S] * v[160 * KQ_S]) - (r[219 * KQ_S] * v[135 * KQ_S]);
    vdot[136 * KQ_S] = 0.0 - (r[176 * KQ_S] * v[136 * KQ_S]) + (r[182 * KQ_S] * v[140 * KQ_S] * v[155 * KQ_S]) + (r[197 * KQ_S] * v[105 * KQ_S] * v[160 * KQ_S]) - (r[198 * KQ_S] * v[136 * KQ_S] * v[160 * KQ_S]) + 0x1.b333340000000p-1 * (r[206 * KQ_S] * v[134 * KQ_S] * v[160 * KQ_S]) - (r[211 * KQ_S] * v[136 * KQ_S]);
    vdot[137 * KQ_S] = 0.0 + (r[46 * KQ_S] * v[141 * KQ_S]) - (r[60 * KQ_S] * v[137 * KQ_S] * v[155 * KQ_S]) - (r[128 * KQ_S] * v[137 * KQ_S]) - (r[249 * KQ_S] * v[137 * KQ_S] * v[160 * KQ_S]);
    vdot[138 * KQ_S] = 0.0 - (r[180 * KQ_S] * v[138 * KQ_S]) + (r[186 * KQ_S] * v[139 * KQ_S] * v[155 * KQ_S]) + (r[193 * KQ_S] * v[104 * KQ_S] * v[160 * KQ_S]) - (r[195 * KQ_S] * v[138 * KQ_S] * v[160 * KQ_S]) - (r[222 * KQ_S] * v[138 * KQ_S]);
    vdot[139 * KQ_S] = 0.0 + (r[180 * KQ_S] * v[138 * KQ_S]) - (r[186 * KQ_S] * v[139 * KQ_S] * v[155 * KQ_S]) - (r[196 * KQ_S] * v[139 * KQ_S] * v[160 * KQ_S]) - (r[223 * KQ_S] * v[139 * KQ_S]);
    vdot[140 * KQ_S] = 0.0 + (r[176 * KQ_S] * v[136 * KQ_S]) - (r[182 * KQ_S] * v[140 * KQ_S] * v[155 * KQ_S]) + (r[195 * KQ_S] * v[138 * KQ_S] * v[160 * KQ_S]) + (r[196 * KQ_S] * v[139 * KQ_S] * v[160 * KQ_S]) - (r[199 * KQ_S] * v[140 * KQ_S] * v[160 * KQ_S]) + 0x1.47ae140000000p-4 * (r[203 * KQ_S] * v[112 * KQ_S] * v[160 * KQ_S]) + 0x1.b333340000000p-1 * (r[207 * KQ_S] * v[135 * KQ_S] * v[160 * KQ_S]) - (r[212 * KQ_S] * v[140 * KQ_S]);
    vdot[141 * KQ_S] = 0.0 + (r[6 * KQ_S] * v[89 * KQ_S]) - (r[22 * KQ_S] * v[141 * KQ_S]) - (r[46 * KQ_S] * v[141 * KQ_S]) + (r[60 * KQ_S] * v[137 * KQ_S] * v[155 * KQ_S]) - (r[101 * KQ_S] * v[141 * KQ_S]) + (r[208 * KQ_S] * v[148 * KQ_S] * v[160 * KQ_S]) - (r[209 * KQ_S] * v[141 * KQ_S] * v[160 * KQ_S]) + (r[254 * KQ_S] * v[147 * KQ_S] * v[160 * KQ_S]);
    vdot[142 * KQ_S] = 0.0 + (r[242 * KQ_S] * v[103 * KQ_S] * f[2 * KQ_S]) - (r[243 * KQ_S] * v[142 * KQ_S] * v[154 * KQ_S]) + -0x1.0000000000000p+1 * (r[244 * KQ_S] * v[142 * KQ_S] * v[142 * KQ_S]) - (r[265 * KQ_S] * v[142 * KQ_S]);
    vdot[143 * KQ_S] = 0.0 + (r[168 * KQ_S] * v[80 * KQ_S]) - (r[173 * KQ_S] * v[143 * KQ_S]) - (r[188 * KQ_S] * v[143 * KQ_S] * f[0 * KQ_S]) + (r[189 * KQ_S] * v[148 * KQ_S]) - (r[224 * KQ_S] * v[143 * KQ_S]) + 0x1.0000000000000p+1 * (r[247 * KQ_S] * v[119 * KQ_S] * v[119 * KQ_S]) - (r[250 * KQ_S] * v[143 * KQ_S] * v[156 * KQ_S]) - (r[251 * KQ_S] * v[143 * KQ_S] * v[159 * KQ_S]) + (r[252 * KQ_S] * v[147 * KQ_S]);
    vdot[144 * KQ_S] = 0.0 + (r[0 * KQ_S] * v[99 * KQ_S]) - (r[16 * KQ_S] * v[144 * KQ_S]) - (r[40 * KQ_S] * v[144 * KQ_S]) + (r[54 * KQ_S] * v[155 * KQ_S] * v[156 * KQ_S]) - (r[69 * KQ_S] * v[144 * KQ_S] * v[157 * KQ_S]) - (r[72 * KQ_S] * v[13 * KQ_S] * v[144 * KQ_S]) - (r[75 * KQ_S] * v[12 * KQ_S] * v[144 * KQ_S]) - (r[78 * KQ_S] * v[12 * KQ_S] * v[13 * KQ_S] * v[144 * KQ_S]) - (r[87 * KQ_S] * v[144 * KQ_S] * v[158 * KQ_S]) - (r[95 * KQ_S] * v[144 * KQ_S]);
}

KQ_HD KQ_NOINLINE void kqu_fun_5(const double* v, const double* f, const double* r, double* vdot)
{
    vdot[145 * KQ_S] = 0.0 + (r[4 * KQ_S] * v[84 * KQ_S]) - (r[20 * KQ_S] * v[145 * KQ_S]) - (r[68 * KQ_S] * v[145 * KQ_S] * v[155 * KQ_S] * v[156 * KQ_S]) + (r[84 * KQ_S] * v[154 * KQ_S] * v[154 * KQ_S]) + (r[85 * KQ_S] * v[150 * KQ_S] * v[154 * KQ_S]) - (r[99 * KQ_S] * v[145 * KQ_S]) - (r[192 * KQ_S] * v[145 * KQ_S]) + (r[232 * KQ_S] * v[160 * KQ_S] * v[160 * KQ_S]) - (r[235 * KQ_S] * v[145 * KQ_S] * v[160 * KQ_S]);
    vdot[146 * KQ_S] = 0.0 + (r[32 * KQ_S] * v[0 * KQ_S]) + (r[42 * KQ_S] * v[106 * KQ_S]) - (r[56 * KQ_S] * v[146 * KQ_S] * v[155 * KQ_S]) + (r[90 * KQ_S] * v[149 * KQ_S] * v[156 * KQ_S]) + (r[92 * KQ_S] * v[151 * KQ_S] * v[157 * KQ_S]) - (r[109 * KQ_S] * v[146 * KQ_S]) - (r[152 * KQ_S] * v[115 * KQ_S] * v[146 * KQ_S]) - (r[231 * KQ_S] * v[146 * KQ_S]) + (r[240 * KQ_S] * v[126 * KQ_S] * v[153 * KQ_S]) + (r[241 * KQ_S] * v[126 * KQ_S] * v[156 * KQ_S]);
    vdot[147 * KQ_S] = 0.0 + (r[250 * KQ_S] * v[143 * KQ_S] * v[156 * KQ_S]) + (r[251 * KQ_S] * v[143 * KQ_S] * v[159 * KQ_S]) - (r[252 * KQ_S] * v[147 * KQ_S]) - (r[253 * KQ_S] * v[147 * KQ_S] * v[152 * KQ_S]) - (r[254 * KQ_S] * v[147 * KQ_S] * v[160 * KQ_S]) - (r[264 * KQ_S] * v[147 * KQ_S]);
    vdot[148 * KQ_S] = 0.0 + (r[188 * KQ_S] * v[143 * KQ_S] * f[0 * KQ_S]) - (r[189 * KQ_S] * v[148 * KQ_S]) + 0x1.3333340000000p-3 * (r[206 * KQ_S] * v[134 * KQ_S] * v[160 * KQ_S]) + 0x1.3333340000000p-3 * (r[207 * KQ_S] * v[135 * KQ_S] * v[160 * KQ_S]) - (r[208 * KQ_S] * v[148 * KQ_S] * v[160 * KQ_S]) - (r[220 * KQ_S] * v[148 * KQ_S]) + (r[253 * KQ_S] * v[147 * KQ_S] * v[152 * KQ_S]);
    vdot[149 * KQ_S] = 0.0 + (r[15 * KQ_S] * v[96 * KQ_S]) - (r[31 * KQ_S] * v[149 * KQ_S]) - (r[53 * KQ_S] * v[149 * KQ_S]) + (r[67 * KQ_S] * v[129 * KQ_S] * v[155 * KQ_S]) - (r[90 * KQ_S] * v[149 * KQ_S] * v[156 * KQ_S]) - (r[136 * KQ_S] * v[149 * KQ_S]) + (r[237 * KQ_S] * v[154 * KQ_S] * v[158 * KQ_S]) - (r[239 * KQ_S] * v[149 * KQ_S]);
    vdot[150 * KQ_S] = 0.0 + (r[51 * KQ_S] * v[154 * KQ_S]) - (r[65 * KQ_S] * v[150 * KQ_S] * v[155 * KQ_S]) - (r[85 * KQ_S] * v[150 * KQ_S] * v[154 * KQ_S]) - (r[86 * KQ_S] * v[150 * KQ_S] * v[157 * KQ_S]) - (r[130 * KQ_S] * v[150 * KQ_S]) - (r[234 * KQ_S] * v[150 * KQ_S] * v[160 * KQ_S]) - (r[238 * KQ_S] * v[150 * KQ_S] * v[158 * KQ_S]);
    vdot[151 * KQ_S] = 0.0 + (r[52 * KQ_S] * v[125 * KQ_S]) - (r[66 * KQ_S] * v[151 * KQ_S] * v[155 * KQ_S]) + 0x1.0000000000000p+1 * (r[87 * KQ_S] * v[144 * KQ_S] * v[158 * KQ_S]) + 0x1.0000000000000p+1 * (r[88 * KQ_S] * v[156 * KQ_S] * v[158 * KQ_S]) + 0x1.0000000000000p+1 * (r[89 * KQ_S] * v[158 * KQ_S] * v[159 * KQ_S]) + (r[91 * KQ_S] * v[129 * KQ_S]) - (r[92 * KQ_S] * v[151 * KQ_S] * v[157 * KQ_S]) - (r[93 * KQ_S] * v[151 * KQ_S] * v[160 * KQ_S]) - (r[134 * KQ_S] * v[151 * KQ_S]);
    vdot[152 * KQ_S] = 0.0 + (r[45 * KQ_S] * v[107 * KQ_S]) + (r[48 * KQ_S] * f[0 * KQ_S]) - (r[59 * KQ_S] * v[108 * KQ_S] * v[152 * KQ_S]) - (r[62 * KQ_S] * v[152 * KQ_S] * v[155 * KQ_S]) + (r[85 * KQ_S] * v[150 * KQ_S] * v[154 * KQ_S]) + (r[86 * KQ_S] * v[150 * KQ_S] * v[157 * KQ_S]) + (r[93 * KQ_S] * v[151 * KQ_S] * v[160 * KQ_S]) - (r[123 * KQ_S] * v[152 * KQ_S]) + (r[202 * KQ_S] * v[130 * KQ_S] * v[160 * KQ_S]) + (r[231 * KQ_S] * v[146 * KQ_S]) + (r[234 * KQ_S] * v[150 * KQ_S] * v[160 * KQ_S]) + (r[249 * KQ_S] * v[137 * KQ_S] * v[160 * KQ_S]) + (r[251 * KQ_S] * v[143 * KQ_S] * v[159 * KQ_S]) - (r[253 * KQ_S] * v[147 * KQ_S] * v[152 * KQ_S]);
}

KQ_HD KQ_NOINLINE void kqu_fun_6(const double* v, const double* f, const double* r, double* vdot)
{
    vdot[153 * KQ_S] = 0.0 + (r[36 * KQ_S] * v[4 * KQ_S]) + (r[50 * KQ_S] * v[123 * KQ_S]) - (r[64 * KQ_S] * v[153 * KQ_S] * v[155 * KQ_S]) + (r[68 * KQ_S] * v[145 * KQ_S] * v[155 * KQ_S] * v[156 * KQ_S]) + (r[69 * KQ_S] * v[144 * KQ_S] * v[157 * KQ_S]) + (r[70 * KQ_S] * v[156 * KQ_S] * v[157 * KQ_S]) + (r[71 * KQ_S] * v[157 * KQ_S] * v[159 * KQ_S]) + (r[72 * KQ_S] * v[13 * KQ_S] * v[144 * KQ_S]) + (r[73 * KQ_S] * v[13 * KQ_S] * v[156 * KQ_S]) + (r[74 * KQ_S] * v[13 * KQ_S] * v[159 * KQ_S]) + (r[75 * KQ_S] * v[12 * KQ_S] * v[144 * KQ_S]) + (r[76 * KQ_S] * v[12 * KQ_S] * v[156 * KQ_S]) + (r[77 * KQ_S] * v[12 * KQ_S] * v[159 * KQ_S]) + (r[78 * KQ_S] * v[12 * KQ_S] * v[13 * KQ_S] * v[144 * KQ_S]) + (r[79 * KQ_S] * v[12 * KQ_S] * v[13 * KQ_S] * v[156 * KQ_S]) + (r[80 * KQ_S] * v[12 * KQ_S] * v[13 * KQ_S] * v[159 * KQ_S]) + (r[81 * KQ_S] * v[120 * KQ_S] * v[155 * KQ_S] * v[156 * KQ_S]) + (r[82 * KQ_S] * v[121 * KQ_S] * v[155 * KQ_S] * v[156 * KQ_S]) + (r[83 * KQ_S] * v[121 * KQ_S] * v[156 * KQ_S]) + (r[87 * KQ_S] * v[144 * KQ_S] * v[158 * KQ_S]) + (r[88 * KQ_S] * v[156 * KQ_S] * v[158 * KQ_S]) + (r[89 * KQ_S] * v[158 * KQ_S] * v[159 * KQ_S]) + (r[90 * KQ_S] * v[149 * KQ_S] * v[156 * KQ_S]) - (r[108 * KQ_S] * v[153 * KQ_S]) - (r[147 * KQ_S] * v[115 * KQ_S] * v[153 * KQ_S]) - (r[151 * KQ_S] * v[115 * KQ_S] * v[153 * KQ_S]) - (r[154 * KQ_S] * v[75 * KQ_S] * v[153 * KQ_S]) - (r[156 * KQ_S] * v[77 * KQ_S] * v[153 * KQ_S]) - (r[240 * KQ_S] * v[126 * KQ_S] * v[153 * KQ_S]) + 0x1.0000000000000p+1 * (r[245 * KQ_S] * v[127 * KQ_S] * v[155 * KQ_S] * v[156 * KQ_S]);
    vdot[154 * KQ_S] = 0.0 + (r[12 * KQ_S] * v[81 * KQ_S]) - (r[28 * KQ_S] * v[154 * KQ_S]) - (r[51 * KQ_S] * v[154 * KQ_S]) + (r[65 * KQ_S] * v[150 * KQ_S] * v[155 * KQ_S]) + -0x1.0000000000000p+1 * (r[84 * KQ_S] * v[154 * KQ_S] * v[154 * KQ_S]) - (r[85 * KQ_S] * v[150 * KQ_S] * v[154 * KQ_S]) - (r[131 * KQ_S] * v[154 * KQ_S]) + (r[193 * KQ_S] * v[104 * KQ_S] * v[160 * KQ_S]) + (r[194 * KQ_S] * v[104 * KQ_S] * v[160 * KQ_S]) + (r[195 * KQ_S] * v[138 * KQ_S] * v[160 * KQ_S]) + (r[196 * KQ_S] * v[139 * KQ_S] * v[160 * KQ_S]) + (r[197 * KQ_S] * v[105 * KQ_S] * v[160 * KQ_S]) + (r[198 * KQ_S] * v[136 * KQ_S] * v[160 * KQ_S]) + (r[199 * KQ_S] * v[140 * KQ_S] * v[160 * KQ_S]) + (r[203 * KQ_S] * v[112 * KQ_S] * v[160 * KQ_S]) + (r[204 * KQ_S] * v[133 * KQ_S] * v[160 * KQ_S]) + (r[205 * KQ_S] * v[132 * KQ_S] * v[160 * KQ_S]) + (r[208 * KQ_S] * v[148 * KQ_S] * v[160 * KQ_S]) + (r[209 * KQ_S] * v[141 * KQ_S] * v[160 * KQ_S]) - (r[233 * KQ_S] * v[154 * KQ_S] * v[160 * KQ_S]) + (r[235 * KQ_S] * v[145 * KQ_S] * v[160 * KQ_S]) - (r[237 * KQ_S] * v[154 * KQ_S] * v[158 * KQ_S]) + (r[239 * KQ_S] * v[149 * KQ_S]) - (r[243 * KQ_S] * v[142 * KQ_S] * v[154 * KQ_S]) + 0x1.0000000000000p+1 * (r[247 * KQ_S] * v[119 * KQ_S] * v[119 * KQ_S]) + (r[249 * KQ_S] * v[137 * KQ_S] * v[160 * KQ_S]) + (r[254 * KQ_S] * v[147 * KQ_S] * v[160 * KQ_S]);
}

KQ_HD KQ_NOINLINE void kqu_fun_7(const double* v, const double* f, const double* r, double* vdot)
{
    vdot[155 * KQ_S] = 0.0 + (r[40 * KQ_S] * v[144 * KQ_S]) + (r[41 * KQ_S] * v[156 * KQ_S]) + (r[42 * KQ_S] * v[106 * KQ_S]) + (r[43 * KQ_S] * v[124 * KQ_S]) + (r[44 * KQ_S] * v[114 * KQ_S]) + (r[46 * KQ_S] * v[141 * KQ_S]) + (r[47 * KQ_S] * v[110 * KQ_S]) + (r[48 * KQ_S] * f[0 * KQ_S]) + (r[49 * KQ_S] * v[109 * KQ_S]) + (r[50 * KQ_S] * v[123 * KQ_S]) + (r[51 * KQ_S] * v[154 * KQ_S]) + (r[52 * KQ_S] * v[125 * KQ_S]) + (r[53 * KQ_S] * v[149 * KQ_S]) - (r[54 * KQ_S] * v[155 * KQ_S] * v[156 * KQ_S]) - (r[55 * KQ_S] * v[155 * KQ_S] * v[159 * KQ_S]) - (r[56 * KQ_S] * v[146 * KQ_S] * v[155 * KQ_S]) - (r[57 * KQ_S] * v[114 * KQ_S] * v[155 * KQ_S]) - (r[58 * KQ_S] * v[113 * KQ_S] * v[155 * KQ_S]) - (r[60 * KQ_S] * v[137 * KQ_S] * v[155 * KQ_S]) - (r[61 * KQ_S] * v[111 * KQ_S] * v[155 * KQ_S]) - (r[62 * KQ_S] * v[152 * KQ_S] * v[155 * KQ_S]) - (r[63 * KQ_S] * v[123 * KQ_S] * v[155 * KQ_S]) - (r[64 * KQ_S] * v[153 * KQ_S] * v[155 * KQ_S]) - (r[65 * KQ_S] * v[150 * KQ_S] * v[155 * KQ_S]) - (r[66 * KQ_S] * v[151 * KQ_S] * v[155 * KQ_S]) - (r[67 * KQ_S] * v[129 * KQ_S] * v[155 * KQ_S]) + (r[68 * KQ_S] * v[145 * KQ_S] * v[155 * KQ_S] * v[156 * KQ_S]) + 0x1.0000000000000p+1 * (r[69 * KQ_S] * v[144 * KQ_S] * v[157 * KQ_S]) + (r[70 * KQ_S] * v[156 * KQ_S] * v[157 * KQ_S]) + 0x1.0000000000000p+1 * (r[72 * KQ_S] * v[13 * KQ_S] * v[144 * KQ_S]) + (r[73 * KQ_S] * v[13 * KQ_S] * v[156 * KQ_S]) + 0x1.0000000000000p+1 * (r[75 * KQ_S] * v[12 * KQ_S] * v[144 * KQ_S]) + (r[76 * KQ_S] * v[12 * KQ_S] * v[156 * KQ_S]) + 0x1.0000000000000p+1 * (r[78 * KQ_S] * v[12 * KQ_S] * v[13 * KQ_S] * v[144 * KQ_S]) + (r[79 * KQ_S] * v[12 * KQ_S] * v[13 * KQ_S] * v[156 * KQ_S]) + (r[81 * KQ_S] * v[120 * KQ_S] * v[155 * KQ_S] * v[156 * KQ_S]) + (r[82 * KQ_S] * v[121 * KQ_S] * v[155 * KQ_S] * v[156 * KQ_S]) + (r[83 * KQ_S] * v[121 * KQ_S] * v[156 * KQ_S]) + 0x1.0000000000000p+2 * (r[87 * KQ_S] * v[144 * KQ_S] * v[158 * KQ_S]) + 0x1.8000000000000p+1 * (r[88 * KQ_S] * v[156 * KQ_S] * v[158 * KQ_S]) + 0x1.0000000000000p+1 * (r[89 * KQ_S] * v[158 * KQ_S] * v[159 * KQ_S]) + 0x1.0000000000000p+1 * (r[90 * KQ_S] * v[149 * KQ_S] * v[156 * KQ_S]) - (r[122 * KQ_S] * v[155 * KQ_S]) + (r[176 * KQ_S] * v[136 * KQ_S]) + (r[177 * KQ_S] * v[128 * KQ_S]) + (r[178 * KQ_S] * v[131 * KQ_S]) + (r[179 * KQ_S] * v[133 * KQ_S]) + (r[180 * KQ_S] * v[138 * KQ_S]) + (r[181 * KQ_S] * v[134 * KQ_S]) - (r[182 * KQ_S] * v[140 * KQ_S] * v[155 * KQ_S]) - (r[183 * KQ_S] * v[131 * KQ_S] * v[155 * KQ_S]) - (r[184 * KQ_S] * v[130 * KQ_S] * v[155 * KQ_S]) - (r[185 * KQ_S] * v[132 * KQ_S] * v[155 * KQ_S]) - (r[186 * KQ_S] * v[139 * KQ_S] * v[155 * KQ_S]) - (r[187 * KQ_S] * v[135 * KQ_S] * v[155 * KQ_S]) + (r[195 * KQ_S] * v[138 * KQ_S] * v[160 * KQ_S]) + (r[241 * KQ_S] * v[126 * KQ_S] * v[156 * KQ_S]) + 0x1.0000000000000p+1 * (r[245 * KQ_S] * v[127 * KQ_S] * v[155 * KQ_S] * v[156 * KQ_S]);
}

KQ_HD KQ_NOINLINE void kqu_fun_8(const double* v, const double* f, const double* r, double* vdot)
{
    vdot[156 * KQ_S] = 0.0 + (r[40 * KQ_S] * v[144 * KQ_S]) - (r[41 * KQ_S] * v[156 * KQ_S]) - (r[54 * KQ_S] * v[155 * KQ_S] * v[156 * KQ_S]) + (r[55 * KQ_S] * v[155 * KQ_S] * v[159 * KQ_S]) - (r[68 * KQ_S] * v[145 * KQ_S] * v[155 * KQ_S] * v[156 * KQ_S]) - (r[70 * KQ_S] * v[156 * KQ_S] * v[157 * KQ_S]) - (r[73 * KQ_S] * v[13 * KQ_S] * v[156 * KQ_S]) - (r[76 * KQ_S] * v[12 * KQ_S] * v[156 * KQ_S]) - (r[79 * KQ_S] * v[12 * KQ_S] * v[13 * KQ_S] * v[156 * KQ_S]) - (r[81 * KQ_S] * v[120 * KQ_S] * v[155 * KQ_S] * v[156 * KQ_S]) - (r[82 * KQ_S] * v[121 * KQ_S] * v[155 * KQ_S] * v[156 * KQ_S]) - (r[83 * KQ_S] * v[121 * KQ_S] * v[156 * KQ_S]) - (r[88 * KQ_S] * v[156 * KQ_S] * v[158 * KQ_S]) - (r[90 * KQ_S] * v[149 * KQ_S] * v[156 * KQ_S]) - (r[124 * KQ_S] * v[156 * KQ_S]) - (r[236 * KQ_S] * v[156 * KQ_S] * v[160 * KQ_S]) - (r[241 * KQ_S] * v[126 * KQ_S] * v[156 * KQ_S]) - (r[245 * KQ_S] * v[127 * KQ_S] * v[155 * KQ_S] * v[156 * KQ_S]) - (r[248 * KQ_S] * v[119 * KQ_S] * v[156 * KQ_S]) - (r[250 * KQ_S] * v[143 * KQ_S] * v[156 * KQ_S]) + (r[252 * KQ_S] * v[147 * KQ_S]) + (r[254 * KQ_S] * v[147 * KQ_S] * v[160 * KQ_S]);
    vdot[157 * KQ_S] = 0.0 + (r[5 * KQ_S] * v[88 * KQ_S]) - (r[21 * KQ_S] * v[157 * KQ_S]) - (r[69 * KQ_S] * v[144 * KQ_S] * v[157 * KQ_S]) - (r[70 * KQ_S] * v[156 * KQ_S] * v[157 * KQ_S]) - (r[71 * KQ_S] * v[157 * KQ_S] * v[159 * KQ_S]) - (r[86 * KQ_S] * v[150 * KQ_S] * v[157 * KQ_S]) - (r[92 * KQ_S] * v[151 * KQ_S] * v[157 * KQ_S]) - (r[100 * KQ_S] * v[157 * KQ_S]);
    vdot[158 * KQ_S] = 0.0 + (r[13 * KQ_S] * v[95 * KQ_S]) - (r[29 * KQ_S] * v[158 * KQ_S]) + -0x1.0000000000000p+1 * (r[87 * KQ_S] * v[144 * KQ_S] * v[158 * KQ_S]) + -0x1.0000000000000p+1 * (r[88 * KQ_S] * v[156 * KQ_S] * v[158 * KQ_S]) + -0x1.0000000000000p+1 * (r[89 * KQ_S] * v[158 * KQ_S] * v[159 * KQ_S]) + (r[93 * KQ_S] * v[151 * KQ_S] * v[160 * KQ_S]) + (r[94 * KQ_S] * v[125 * KQ_S] * v[160 * KQ_S]) - (r[132 * KQ_S] * v[158 * KQ_S]) + (r[231 * KQ_S] * v[146 * KQ_S]) - (r[237 * KQ_S] * v[154 * KQ_S] * v[158 * KQ_S]) - (r[238 * KQ_S] * v[150 * KQ_S] * v[158 * KQ_S]) + (r[239 * KQ_S] * v[149 * KQ_S]);
    vdot[159 * KQ_S] = 0.0 + (r[41 * KQ_S] * v[156 * KQ_S]) - (r[55 * KQ_S] * v[155 * KQ_S] * v[159 * KQ_S]) - (r[71 * KQ_S] * v[157 * KQ_S] * v[159 * KQ_S]) - (r[74 * KQ_S] * v[13 * KQ_S] * v[159 * KQ_S]) - (r[77 * KQ_S] * v[12 * KQ_S] * v[159 * KQ_S]) - (r[80 * KQ_S] * v[12 * KQ_S] * v[13 * KQ_S] * v[159 * KQ_S]) - (r[89 * KQ_S] * v[158 * KQ_S] * v[159 * KQ_S]) - (r[125 * KQ_S] * v[159 * KQ_S]) - (r[251 * KQ_S] * v[143 * KQ_S] * v[159 * KQ_S]) + (r[253 * KQ_S] * v[147 * KQ_S] * v[152 * KQ_S]);
}

KQ_HD KQ_NOINLINE void kqu_fun_9(const double* v, const double* f, const double* r, double* vdot)
{
    vdot[160 * KQ_S] = 0.0 + (r[86 * KQ_S] * v[150 * KQ_S] * v[157 * KQ_S]) - (r[93 * KQ_S] * v[151 * KQ_S] * v[160 * KQ_S]) - (r[94 * KQ_S] * v[125 * KQ_S] * v[160 * KQ_S]) + (r[137 * KQ_S] * f[1 * KQ_S]) - (r[138 * KQ_S] * v[160 * KQ_S]) - (r[139 * KQ_S] * v[160 * KQ_S]) + 0x1.0000000000000p+1 * (r[192 * KQ_S] * v[145 * KQ_S]) - (r[193 * KQ_S] * v[104 * KQ_S] * v[160 * KQ_S]) - (r[194 * KQ_S] * v[104 * KQ_S] * v[160 * KQ_S]) - (r[195 * KQ_S] * v[138 * KQ_S] * v[160 * KQ_S]) - (r[196 * KQ_S] * v[139 * KQ_S] * v[160 * KQ_S]) - (r[197 * KQ_S] * v[105 * KQ_S] * v[160 * KQ_S]) - (r[198 * KQ_S] * v[136 * KQ_S] * v[160 * KQ_S]) - (r[199 * KQ_S] * v[140 * KQ_S] * v[160 * KQ_S]) + -0x1.0000000000000p+1 * (r[200 * KQ_S] * v[128 * KQ_S] * v[160 * KQ_S]) - (r[201 * KQ_S] * v[131 * KQ_S] * v[160 * KQ_S]) - (r[202 * KQ_S] * v[130 * KQ_S] * v[160 * KQ_S]) - (r[203 * KQ_S] * v[112 * KQ_S] * v[160 * KQ_S]) - (r[204 * KQ_S] * v[133 * KQ_S] * v[160 * KQ_S]) - (r[205 * KQ_S] * v[132 * KQ_S] * v[160 * KQ_S]) - (r[206 * KQ_S] * v[134 * KQ_S] * v[160 * KQ_S]) - (r[207 * KQ_S] * v[135 * KQ_S] * v[160 * KQ_S]) - (r[208 * KQ_S] * v[148 * KQ_S] * v[160 * KQ_S]) - (r[209 * KQ_S] * v[141 * KQ_S] * v[160 * KQ_S]) + (r[231 * KQ_S] * v[146 * KQ_S]) + -0x1.0000000000000p+1 * (r[232 * KQ_S] * v[160 * KQ_S] * v[160 * KQ_S]) - (r[233 * KQ_S] * v[154 * KQ_S] * v[160 * KQ_S]) - (r[234 * KQ_S] * v[150 * KQ_S] * v[160 * KQ_S]) - (r[235 * KQ_S] * v[145 * KQ_S] * v[160 * KQ_S]) - (r[236 * KQ_S] * v[156 * KQ_S] * v[160 * KQ_S]) + (r[246 * KQ_S] * v[122 * KQ_S] * f[0 * KQ_S]) - (r[249 * KQ_S] * v[137 * KQ_S] * v[160 * KQ_S]) - (r[254 * KQ_S] * v[147 * KQ_S] * v[160 * KQ_S]);
}

KQ_HD inline void kqu_fun(const double* v, const double* f, const double* r, double* vdot)
{
    kqu_fun_0(v, f, r, vdot);
    kqu_fun_1(v, f, r, vdot);
    kqu_fun_2(v, f, r, vdot);
    kqu_fun_3(v, f, r, vdot);
    kqu_fun_4(v, f, r, vdot);
    kqu_fun_5(v, f, r, vdot);
    kqu_fun_6(v, f, r, vdot);
    kqu_fun_7(v, f, r, vdot);
    kqu_fun_8(v, f, r, vdot);
    kqu_fun_9(v, f, r, vdot);
}

KQ_HD KQ_NOINLINE void kqu_jac_0(const double* v, const double* f, const double* r, double* jvs)
{
    jvs[0 * KQ_S] = 0.0 - (r[32 * KQ_S]);
    jvs[1 * KQ_S] = 0.0 - (r[33 * KQ_S]);
    jvs[2 * KQ_S] = 0.0 - (r[34 * KQ_S]);
    jvs[3 * KQ_S] = 0.0 - (r[35 * KQ_S]);
    jvs[4 * KQ_S] = 0.0 - (r[36 * KQ_S]);
    jvs[5 * KQ_S] = 0.0 - (r[37 * KQ_S]);
    jvs[6 * KQ_S] = 0.0 - (r[38 * KQ_S]);
    jvs[7 * KQ_S] = 0.0 - (r[39 * KQ_S]);
    jvs[8 * KQ_S] = 0.0 + (r[39 * KQ_S]);
    jvs[9 * KQ_S] = 0.0 - (r[112 * KQ_S]);
    jvs[10 * KQ_S] = 0.0 + (r[37 * KQ_S]);
    jvs[11 * KQ_S] = 0.0 - (r[113 * KQ_S]);
    jvs[12 * KQ_S] = 0.0 - (r[114 * KQ_S]);
    jvs[13 * KQ_S] = 0.0 + (r[38 * KQ_S]);
    jvs[14 * KQ_S] = 0.0 - (r[115 * KQ_S]);
    jvs[15 * KQ_S] = 0.0 - (r[120 * KQ_S]);
    jvs[16 * KQ_S] = 0.0 - (r[121 * KQ_S]);
    jvs[17 * KQ_S] = 0.0 - (r[116 * KQ_S]);
    jvs[18 * KQ_S] = 0.0 - (r[117 * KQ_S]);
    jvs[19 * KQ_S] = 0.0 - (r[118 * KQ_S]);
    jvs[20 * KQ_S] = 0.0 + (r[35 * KQ_S]);
    jvs[21 * KQ_S] = 0.0 - (r[119 * KQ_S]);
    jvs[22 * KQ_S] = 0.0;
    jvs[23 * KQ_S] = 0.0 + (r[263 * KQ_S]);
    jvs[24 * KQ_S] = 0.0 + (r[262 * KQ_S]);
    jvs[25 * KQ_S] = 0.0 + (r[266 * KQ_S]);
    jvs[26 * KQ_S] = 0.0 + (r[265 * KQ_S]);
    jvs[27 * KQ_S] = 0.0 + (r[95 * KQ_S]);
    jvs[28 * KQ_S] = 0.0 + (r[264 * KQ_S]);
    jvs[29 * KQ_S] = 0.0 + (r[124 * KQ_S]);
    jvs[30 * KQ_S] = 0.0 + (r[125 * KQ_S]);
    jvs[31 * KQ_S] = 0.0;
    jvs[32 * KQ_S] = 0.0 + (r[96 * KQ_S]);
    jvs[33 * KQ_S] = 0.0;
    jvs[34 * KQ_S] = 0.0 + (r[267 * KQ_S]);
    jvs[35 * KQ_S] = 0.0 + (r[127 * KQ_S]);
    jvs[36 * KQ_S] = 0.0 + (r[126 * KQ_S]);
    jvs[37 * KQ_S] = 0.0 + (r[97 * KQ_S]);
    jvs[38 * KQ_S] = 0.0 - (r[267 * KQ_S]);
    jvs[39 * KQ_S] = 0.0 + (r[202 * KQ_S] * v[160 * KQ_S]);
    jvs[40 * KQ_S] = 0.0 + (r[201 * KQ_S] * v[160 * KQ_S]);
    jvs[41 * KQ_S] = 0.0 + (r[201 * KQ_S] * v[131 * KQ_S]) + (r[202 * KQ_S] * v[130 * KQ_S]);
    jvs[42 * KQ_S] = 0.0;
    jvs[43 * KQ_S] = 0.0 + (r[98 * KQ_S]);
    jvs[44 * KQ_S] = 0.0;
    jvs[45 * KQ_S] = 0.0 + (r[99 * KQ_S]);
    jvs[46 * KQ_S] = 0.0;
    jvs[47 * KQ_S] = 0.0 + (r[100 * KQ_S]);
    jvs[48 * KQ_S] = 0.0;
    jvs[49 * KQ_S] = 0.0 + (r[128 * KQ_S]);
    jvs[50 * KQ_S] = 0.0 + (r[101 * KQ_S]);
    jvs[51 * KQ_S] = 0.0;
    jvs[52 * KQ_S] = 0.0 + (r[102 * KQ_S]);
    jvs[53 * KQ_S] = 0.0;
    jvs[54 * KQ_S] = 0.0 + (r[103 * KQ_S]);
    jvs[55 * KQ_S] = 0.0;
    jvs[56 * KQ_S] = 0.0 + (r[104 * KQ_S]);
    jvs[57 * KQ_S] = 0.0 + (r[129 * KQ_S]);
    jvs[58 * KQ_S] = 0.0 + (r[108 * KQ_S]);
    jvs[59 * KQ_S] = 0.0;
    jvs[60 * KQ_S] = 0.0 + (r[105 * KQ_S]);
    jvs[61 * KQ_S] = 0.0;
    jvs[62 * KQ_S] = 0.0 + (r[106 * KQ_S]);
    jvs[63 * KQ_S] = 0.0;
    jvs[64 * KQ_S] = 0.0 + (r[107 * KQ_S]);
    jvs[65 * KQ_S] = 0.0;
    jvs[66 * KQ_S] = 0.0 + (r[139 * KQ_S]);
    jvs[67 * KQ_S] = 0.0;
    jvs[68 * KQ_S] = 0.0 + (r[109 * KQ_S]);
    jvs[69 * KQ_S] = 0.0;
    jvs[70 * KQ_S] = 0.0 + (r[110 * KQ_S]);
    jvs[71 * KQ_S] = 0.0;
    jvs[72 * KQ_S] = 0.0 + (r[111 * KQ_S]);
    jvs[73 * KQ_S] = 0.0 + (r[112 * KQ_S]);
    jvs[74 * KQ_S] = 0.0;
    jvs[75 * KQ_S] = 0.0 + (r[120 * KQ_S]);
    jvs[76 * KQ_S] = 0.0;
    jvs[77 * KQ_S] = 0.0 + (r[121 * KQ_S]);
    jvs[78 * KQ_S] = 0.0;
    jvs[79 * KQ_S] = 0.0 + (r[113 * KQ_S]);
    jvs[80 * KQ_S] = 0.0;
    jvs[81 * KQ_S] = 0.0 + (r[114 * KQ_S]);
    jvs[82 * KQ_S] = 0.0;
    jvs[83 * KQ_S] = 0.0 + (r[115 * KQ_S]);
    jvs[84 * KQ_S] = 0.0;
    jvs[85 * KQ_S] = 0.0;
    jvs[86 * KQ_S] = 0.0 + (r[122 * KQ_S]);
    jvs[87 * KQ_S] = 0.0 + (r[116 * KQ_S]);
    jvs[88 * KQ_S] = 0.0;
    jvs[89 * KQ_S] = 0.0 + (r[117 * KQ_S]);
    jvs[90 * KQ_S] = 0.0;
    jvs[91 * KQ_S] = 0.0 + (r[118 * KQ_S]);
    jvs[92 * KQ_S] = 0.0;
    jvs[93 * KQ_S] = 0.0 + (r[119 * KQ_S]);
    jvs[94 * KQ_S] = 0.0;
    jvs[95 * KQ_S] = 0.0;
    jvs[96 * KQ_S] = 0.0 + (r[132 * KQ_S]);
    jvs[97 * KQ_S] = 0.0;
    jvs[98 * KQ_S] = 0.0 + (r[133 * KQ_S]);
    jvs[99 * KQ_S] = 0.0 + (r[134 * KQ_S]);
    jvs[100 * KQ_S] = 0.0;
    jvs[101 * KQ_S] = 0.0 + (r[135 * KQ_S]);
    jvs[102 * KQ_S] = 0.0 + (r[136 * KQ_S]);
    jvs[103 * KQ_S] = 0.0;
    jvs[104 * KQ_S] = 0.0 + (r[157 * KQ_S]);
    jvs[105 * KQ_S] = 0.0;
    jvs[106 * KQ_S] = 0.0 + (r[165 * KQ_S]);
    jvs[107 * KQ_S] = 0.0 + (r[158 * KQ_S]);
    jvs[108 * KQ_S] = 0.0 - (r[165 * KQ_S]);
    jvs[109 * KQ_S] = 0.0 + (r[150 * KQ_S] * f[0 * KQ_S]) + (r[151 * KQ_S] * v[153 * KQ_S]) + (r[152 * KQ_S] * v[146 * KQ_S]);
    jvs[110 * KQ_S] = 0.0 + (r[152 * KQ_S] * v[115 * KQ_S]);
}

KQ_HD KQ_NOINLINE void kqu_jac_1(const double* v, const double* f, const double* r, double* jvs)
{
    jvs[111 * KQ_S] = 0.0 + (r[151 * KQ_S] * v[115 * KQ_S]);
    jvs[112 * KQ_S] = 0.0;
    jvs[113 * KQ_S] = 0.0 + (r[159 * KQ_S]);
    jvs[114 * KQ_S] = 0.0;
    jvs[115 * KQ_S] = 0.0 + (r[160 * KQ_S]);
    jvs[116 * KQ_S] = 0.0 - (r[160 * KQ_S]);
    jvs[117 * KQ_S] = 0.0 + (r[148 * KQ_S] * v[115 * KQ_S]);
    jvs[118 * KQ_S] = 0.0 + (r[149 * KQ_S] * v[115 * KQ_S]);
    jvs[119 * KQ_S] = 0.0 + (r[148 * KQ_S] * v[101 * KQ_S]) + (r[149 * KQ_S] * v[102 * KQ_S]);
    jvs[120 * KQ_S] = 0.0;
    jvs[121 * KQ_S] = 0.0 + (r[161 * KQ_S]);
    jvs[122 * KQ_S] = 0.0;
    jvs[123 * KQ_S] = 0.0 + (r[162 * KQ_S]);
    jvs[124 * KQ_S] = 0.0;
    jvs[125 * KQ_S] = 0.0 + (r[163 * KQ_S]);
    jvs[126 * KQ_S] = 0.0 - (r[163 * KQ_S]);
    jvs[127 * KQ_S] = 0.0 + (r[153 * KQ_S] * f[0 * KQ_S]);
    jvs[128 * KQ_S] = 0.0 + (r[155 * KQ_S] * f[0 * KQ_S]);
    jvs[129 * KQ_S] = 0.0;
    jvs[130 * KQ_S] = 0.0 + (r[164 * KQ_S]);
    jvs[131 * KQ_S] = 0.0 - (r[164 * KQ_S]);
    jvs[132 * KQ_S] = 0.0 + (r[154 * KQ_S] * v[153 * KQ_S]);
    jvs[133 * KQ_S] = 0.0 + (r[156 * KQ_S] * v[153 * KQ_S]);
    jvs[134 * KQ_S] = 0.0 + (r[154 * KQ_S] * v[75 * KQ_S]) + (r[156 * KQ_S] * v[77 * KQ_S]);
    jvs[135 * KQ_S] = 0.0;
    jvs[136 * KQ_S] = 0.0 + (r[211 * KQ_S]);
    jvs[137 * KQ_S] = 0.0 + (r[212 * KQ_S]);
    jvs[138 * KQ_S] = 0.0;
    jvs[139 * KQ_S] = 0.0 + (r[213 * KQ_S]);
    jvs[140 * KQ_S] = 0.0 + (r[215 * KQ_S]);
    jvs[141 * KQ_S] = 0.0 + (r[214 * KQ_S]);
    jvs[142 * KQ_S] = 0.0;
    jvs[143 * KQ_S] = 0.0 + (r[217 * KQ_S]);
    jvs[144 * KQ_S] = 0.0 + (r[216 * KQ_S]);
    jvs[145 * KQ_S] = 0.0;
    jvs[146 * KQ_S] = 0.0 + (r[218 * KQ_S]);
    jvs[147 * KQ_S] = 0.0 + (r[219 * KQ_S]);
    jvs[148 * KQ_S] = 0.0;
    jvs[149 * KQ_S] = 0.0 + (r[224 * KQ_S]);
    jvs[150 * KQ_S] = 0.0 + (r[264 * KQ_S]);
    jvs[151 * KQ_S] = 0.0 + (r[220 * KQ_S]);
    jvs[152 * KQ_S] = 0.0;
    jvs[153 * KQ_S] = 0.0 + (r[130 * KQ_S]);
    jvs[154 * KQ_S] = 0.0 + (r[131 * KQ_S]);
    jvs[155 * KQ_S] = 0.0;
    jvs[156 * KQ_S] = 0.0 + (r[221 * KQ_S]);
    jvs[157 * KQ_S] = 0.0;
    jvs[158 * KQ_S] = 0.0 + (r[222 * KQ_S]);
    jvs[159 * KQ_S] = 0.0 + (r[223 * KQ_S]);
    jvs[160 * KQ_S] = 0.0;
    jvs[161 * KQ_S] = 0.0 + (r[226 * KQ_S]);
    jvs[162 * KQ_S] = 0.0 + (r[268 * KQ_S]);
    jvs[163 * KQ_S] = 0.0 + (r[225 * KQ_S]);
    jvs[164 * KQ_S] = 0.0;
    jvs[165 * KQ_S] = 0.0 + (r[260 * KQ_S]);
    jvs[166 * KQ_S] = 0.0;
    jvs[167 * KQ_S] = 0.0 + (r[261 * KQ_S]);
    jvs[168 * KQ_S] = 0.0 - (r[14 * KQ_S]);
    jvs[169 * KQ_S] = 0.0 + (r[30 * KQ_S]);
    jvs[170 * KQ_S] = 0.0 - (r[141 * KQ_S]);
    jvs[171 * KQ_S] = 0.0 + (r[144 * KQ_S]);
    jvs[172 * KQ_S] = 0.0 + (r[141 * KQ_S]);
    jvs[173 * KQ_S] = 0.0 - (r[144 * KQ_S]) - (r[153 * KQ_S] * f[0 * KQ_S]) - (r[154 * KQ_S] * v[153 * KQ_S]) - (r[161 * KQ_S]);
    jvs[174 * KQ_S] = 0.0 - (r[154 * KQ_S] * v[75 * KQ_S]);
    jvs[175 * KQ_S] = 0.0 - (r[142 * KQ_S]);
    jvs[176 * KQ_S] = 0.0 + (r[145 * KQ_S]);
    jvs[177 * KQ_S] = 0.0 + (r[142 * KQ_S]);
    jvs[178 * KQ_S] = 0.0 - (r[145 * KQ_S]) - (r[155 * KQ_S] * f[0 * KQ_S]) - (r[156 * KQ_S] * v[153 * KQ_S]) - (r[162 * KQ_S]);
    jvs[179 * KQ_S] = 0.0 - (r[156 * KQ_S] * v[77 * KQ_S]);
    jvs[180 * KQ_S] = 0.0 - (r[166 * KQ_S]);
    jvs[181 * KQ_S] = 0.0 + (r[171 * KQ_S]);
    jvs[182 * KQ_S] = 0.0 - (r[167 * KQ_S]);
    jvs[183 * KQ_S] = 0.0 + (r[172 * KQ_S]);
    jvs[184 * KQ_S] = 0.0 - (r[168 * KQ_S]);
    jvs[185 * KQ_S] = 0.0 + (r[173 * KQ_S]);
    jvs[186 * KQ_S] = 0.0 - (r[12 * KQ_S]);
    jvs[187 * KQ_S] = 0.0 + (r[28 * KQ_S]);
    jvs[188 * KQ_S] = 0.0 - (r[170 * KQ_S]);
    jvs[189 * KQ_S] = 0.0 + (r[175 * KQ_S]);
    jvs[190 * KQ_S] = 0.0 - (r[169 * KQ_S]);
    jvs[191 * KQ_S] = 0.0 + (r[174 * KQ_S]);
    jvs[192 * KQ_S] = 0.0 - (r[4 * KQ_S]);
    jvs[193 * KQ_S] = 0.0 + (r[20 * KQ_S]);
    jvs[194 * KQ_S] = 0.0 - (r[1 * KQ_S]);
    jvs[195 * KQ_S] = 0.0 + (r[17 * KQ_S]);
    jvs[196 * KQ_S] = 0.0 - (r[2 * KQ_S]);
    jvs[197 * KQ_S] = 0.0 + (r[18 * KQ_S]);
    jvs[198 * KQ_S] = 0.0 - (r[3 * KQ_S]);
    jvs[199 * KQ_S] = 0.0 + (r[19 * KQ_S]);
    jvs[200 * KQ_S] = 0.0 - (r[5 * KQ_S]);
    jvs[201 * KQ_S] = 0.0 + (r[21 * KQ_S]);
    jvs[202 * KQ_S] = 0.0 - (r[6 * KQ_S]);
    jvs[203 * KQ_S] = 0.0 + (r[22 * KQ_S]);
    jvs[204 * KQ_S] = 0.0 - (r[7 * KQ_S]);
    jvs[205 * KQ_S] = 0.0 + (r[23 * KQ_S]);
    jvs[206 * KQ_S] = 0.0 - (r[8 * KQ_S]);
}

KQ_HD KQ_NOINLINE void kqu_jac_2(const double* v, const double* f, const double* r, double* jvs)
{
    jvs[207 * KQ_S] = 0.0 + (r[24 * KQ_S]);
    jvs[208 * KQ_S] = 0.0 - (r[9 * KQ_S]);
    jvs[209 * KQ_S] = 0.0 + (r[25 * KQ_S]);
    jvs[210 * KQ_S] = 0.0 - (r[10 * KQ_S]);
    jvs[211 * KQ_S] = 0.0 + (r[26 * KQ_S]);
    jvs[212 * KQ_S] = 0.0 - (r[11 * KQ_S]);
    jvs[213 * KQ_S] = 0.0 + (r[27 * KQ_S]);
    jvs[214 * KQ_S] = 0.0 - (r[13 * KQ_S]);
    jvs[215 * KQ_S] = 0.0 + (r[29 * KQ_S]);
    jvs[216 * KQ_S] = 0.0 - (r[15 * KQ_S]);
    jvs[217 * KQ_S] = 0.0 + (r[31 * KQ_S]);
    jvs[218 * KQ_S] = 0.0 - (r[227 * KQ_S]);
    jvs[219 * KQ_S] = 0.0 + (r[229 * KQ_S]);
    jvs[220 * KQ_S] = 0.0 - (r[228 * KQ_S]);
    jvs[221 * KQ_S] = 0.0 + (r[230 * KQ_S]);
    jvs[222 * KQ_S] = 0.0 - (r[0 * KQ_S]);
    jvs[223 * KQ_S] = 0.0 + (r[16 * KQ_S]);
    jvs[224 * KQ_S] = 0.0 - (r[140 * KQ_S]);
    jvs[225 * KQ_S] = 0.0 + (r[143 * KQ_S]);
    jvs[226 * KQ_S] = 0.0 - (r[148 * KQ_S] * v[115 * KQ_S]) - (r[158 * KQ_S]);
    jvs[227 * KQ_S] = 0.0 + (r[146 * KQ_S] * f[0 * KQ_S]) - (r[148 * KQ_S] * v[101 * KQ_S]);
    jvs[228 * KQ_S] = 0.0 - (r[149 * KQ_S] * v[115 * KQ_S]) - (r[159 * KQ_S]);
    jvs[229 * KQ_S] = 0.0 + (r[147 * KQ_S] * v[153 * KQ_S]) - (r[149 * KQ_S] * v[102 * KQ_S]);
    jvs[230 * KQ_S] = 0.0 + (r[147 * KQ_S] * v[115 * KQ_S]);
    jvs[231 * KQ_S] = 0.0 - (r[242 * KQ_S] * f[2 * KQ_S]) - (r[263 * KQ_S]);
    jvs[232 * KQ_S] = 0.0 + (r[248 * KQ_S] * v[156 * KQ_S]);
    jvs[233 * KQ_S] = 0.0 + (r[241 * KQ_S] * v[156 * KQ_S]);
    jvs[234 * KQ_S] = 0.0 + (r[236 * KQ_S] * v[160 * KQ_S]) + (r[241 * KQ_S] * v[126 * KQ_S]) + (r[248 * KQ_S] * v[119 * KQ_S]);
    jvs[235 * KQ_S] = 0.0 + (r[236 * KQ_S] * v[156 * KQ_S]);
    jvs[236 * KQ_S] = 0.0 + (r[166 * KQ_S]);
    jvs[237 * KQ_S] = 0.0 - (r[171 * KQ_S]) - (r[193 * KQ_S] * v[160 * KQ_S]) - (r[194 * KQ_S] * v[160 * KQ_S]) - (r[221 * KQ_S]);
    jvs[238 * KQ_S] = 0.0 - (r[193 * KQ_S] * v[104 * KQ_S]) - (r[194 * KQ_S] * v[104 * KQ_S]);
    jvs[239 * KQ_S] = 0.0 + (r[10 * KQ_S]);
    jvs[240 * KQ_S] = 0.0 + (r[194 * KQ_S] * v[160 * KQ_S]);
    jvs[241 * KQ_S] = 0.0 - (r[26 * KQ_S]) - (r[106 * KQ_S]) - (r[197 * KQ_S] * v[160 * KQ_S]);
    jvs[242 * KQ_S] = 0.0 + (r[194 * KQ_S] * v[104 * KQ_S]) - (r[197 * KQ_S] * v[105 * KQ_S]);
    jvs[243 * KQ_S] = 0.0 + (r[1 * KQ_S]);
    jvs[244 * KQ_S] = 0.0 - (r[17 * KQ_S]) - (r[42 * KQ_S]) - (r[96 * KQ_S]);
    jvs[245 * KQ_S] = 0.0 + (r[56 * KQ_S] * v[155 * KQ_S]);
    jvs[246 * KQ_S] = 0.0 + (r[56 * KQ_S] * v[146 * KQ_S]);
    jvs[247 * KQ_S] = 0.0 + (r[3 * KQ_S]);
    jvs[248 * KQ_S] = 0.0 - (r[19 * KQ_S]) - (r[45 * KQ_S]) - (r[98 * KQ_S]);
    jvs[249 * KQ_S] = 0.0 + (r[59 * KQ_S] * v[152 * KQ_S]);
    jvs[250 * KQ_S] = 0.0 + (r[59 * KQ_S] * v[108 * KQ_S]);
    jvs[251 * KQ_S] = 0.0 + (r[33 * KQ_S]);
    jvs[252 * KQ_S] = 0.0 + (r[45 * KQ_S]);
    jvs[253 * KQ_S] = 0.0 - (r[59 * KQ_S] * v[152 * KQ_S]) - (r[110 * KQ_S]);
    jvs[254 * KQ_S] = 0.0 - (r[59 * KQ_S] * v[108 * KQ_S]);
    jvs[255 * KQ_S] = 0.0 - (r[49 * KQ_S]) - (r[104 * KQ_S]);
    jvs[256 * KQ_S] = 0.0 + (r[63 * KQ_S] * v[155 * KQ_S]);
    jvs[257 * KQ_S] = 0.0 + (r[63 * KQ_S] * v[123 * KQ_S]);
    jvs[258 * KQ_S] = 0.0 + (r[9 * KQ_S]);
    jvs[259 * KQ_S] = 0.0 - (r[25 * KQ_S]) - (r[47 * KQ_S]) - (r[105 * KQ_S]);
    jvs[260 * KQ_S] = 0.0 + (r[61 * KQ_S] * v[155 * KQ_S]);
    jvs[261 * KQ_S] = 0.0 + (r[61 * KQ_S] * v[111 * KQ_S]);
    jvs[262 * KQ_S] = 0.0 + (r[34 * KQ_S]);
    jvs[263 * KQ_S] = 0.0 + (r[47 * KQ_S]);
    jvs[264 * KQ_S] = 0.0 - (r[61 * KQ_S] * v[155 * KQ_S]) - (r[111 * KQ_S]);
    jvs[265 * KQ_S] = 0.0 - (r[61 * KQ_S] * v[111 * KQ_S]);
    jvs[266 * KQ_S] = 0.0 + (r[11 * KQ_S]);
    jvs[267 * KQ_S] = 0.0 - (r[27 * KQ_S]) - (r[107 * KQ_S]) - (r[203 * KQ_S] * v[160 * KQ_S]);
    jvs[268 * KQ_S] = 0.0 - (r[203 * KQ_S] * v[112 * KQ_S]);
    jvs[269 * KQ_S] = 0.0 - (r[58 * KQ_S] * v[155 * KQ_S]) - (r[127 * KQ_S]);
    jvs[270 * KQ_S] = 0.0 + (r[44 * KQ_S]);
    jvs[271 * KQ_S] = 0.0 - (r[58 * KQ_S] * v[113 * KQ_S]);
    jvs[272 * KQ_S] = 0.0 + (r[58 * KQ_S] * v[155 * KQ_S]);
}

KQ_HD KQ_NOINLINE void kqu_jac_3(const double* v, const double* f, const double* r, double* jvs)
{
    jvs[273 * KQ_S] = 0.0 - (r[44 * KQ_S]) - (r[57 * KQ_S] * v[155 * KQ_S]) - (r[126 * KQ_S]);
    jvs[274 * KQ_S] = 0.0 + (r[43 * KQ_S]);
    jvs[275 * KQ_S] = 0.0 - (r[57 * KQ_S] * v[114 * KQ_S]) + (r[58 * KQ_S] * v[113 * KQ_S]);
    jvs[276 * KQ_S] = 0.0 + (r[140 * KQ_S]);
    jvs[277 * KQ_S] = 0.0 - (r[148 * KQ_S] * v[115 * KQ_S]);
    jvs[278 * KQ_S] = 0.0 - (r[149 * KQ_S] * v[115 * KQ_S]);
    jvs[279 * KQ_S] = 0.0 - (r[143 * KQ_S]) - (r[146 * KQ_S] * f[0 * KQ_S]) - (r[147 * KQ_S] * v[153 * KQ_S]) - (r[148 * KQ_S] * v[101 * KQ_S]) - (r[149 * KQ_S] * v[102 * KQ_S]) - (r[150 * KQ_S] * f[0 * KQ_S]) - (r[151 * KQ_S] * v[153 * KQ_S]) - (r[152 * KQ_S] * v[146 * KQ_S]) - (r[157 * KQ_S]);
    jvs[280 * KQ_S] = 0.0 - (r[152 * KQ_S] * v[115 * KQ_S]);
    jvs[281 * KQ_S] = 0.0 - (r[147 * KQ_S] * v[115 * KQ_S]) - (r[151 * KQ_S] * v[115 * KQ_S]);
    jvs[282 * KQ_S] = 0.0 - (r[191 * KQ_S]) - (r[210 * KQ_S] * v[160 * KQ_S]) - (r[226 * KQ_S]);
    jvs[283 * KQ_S] = 0.0 + (r[258 * KQ_S] * v[152 * KQ_S]);
    jvs[284 * KQ_S] = 0.0 + (r[190 * KQ_S] * f[0 * KQ_S]);
    jvs[285 * KQ_S] = 0.0 + (r[258 * KQ_S] * v[117 * KQ_S]);
    jvs[286 * KQ_S] = 0.0 - (r[210 * KQ_S] * v[116 * KQ_S]);
    jvs[287 * KQ_S] = 0.0 - (r[257 * KQ_S]) - (r[258 * KQ_S] * v[152 * KQ_S]) - (r[259 * KQ_S] * v[160 * KQ_S]) - (r[268 * KQ_S]);
    jvs[288 * KQ_S] = 0.0 + (r[255 * KQ_S] * v[156 * KQ_S]) + (r[256 * KQ_S] * v[159 * KQ_S]);
    jvs[289 * KQ_S] = 0.0 - (r[258 * KQ_S] * v[117 * KQ_S]);
    jvs[290 * KQ_S] = 0.0 + (r[255 * KQ_S] * v[118 * KQ_S]);
    jvs[291 * KQ_S] = 0.0 + (r[256 * KQ_S] * v[118 * KQ_S]);
    jvs[292 * KQ_S] = 0.0 - (r[259 * KQ_S] * v[117 * KQ_S]);
    jvs[293 * KQ_S] = 0.0 + (r[169 * KQ_S]);
    jvs[294 * KQ_S] = 0.0 + (r[191 * KQ_S]);
    jvs[295 * KQ_S] = 0.0 + (r[257 * KQ_S]);
    jvs[296 * KQ_S] = 0.0 - (r[174 * KQ_S]) - (r[190 * KQ_S] * f[0 * KQ_S]) - (r[225 * KQ_S]) - (r[255 * KQ_S] * v[156 * KQ_S]) - (r[256 * KQ_S] * v[159 * KQ_S]);
    jvs[297 * KQ_S] = 0.0;
    jvs[298 * KQ_S] = 0.0 - (r[255 * KQ_S] * v[118 * KQ_S]);
    jvs[299 * KQ_S] = 0.0 - (r[256 * KQ_S] * v[118 * KQ_S]);
    jvs[300 * KQ_S] = 0.0;
    jvs[301 * KQ_S] = 0.0 + (r[228 * KQ_S]);
    jvs[302 * KQ_S] = 0.0 - (r[230 * KQ_S]) + -0x1.0000000000000p+1 * (r[247 * KQ_S] * 0x1.0000000000000p+1 * v[119 * KQ_S]) - (r[248 * KQ_S] * v[156 * KQ_S]) - (r[261 * KQ_S]);
    jvs[303 * KQ_S] = 0.0 - (r[248 * KQ_S] * v[119 * KQ_S]);
    jvs[304 * KQ_S] = 0.0 + (r[7 * KQ_S]);
    jvs[305 * KQ_S] = 0.0 + (r[248 * KQ_S] * v[156 * KQ_S]);
    jvs[306 * KQ_S] = 0.0 - (r[23 * KQ_S]) - (r[81 * KQ_S] * v[155 * KQ_S] * v[156 * KQ_S]) - (r[102 * KQ_S]);
    jvs[307 * KQ_S] = 0.0 - (r[81 * KQ_S] * v[120 * KQ_S] * v[156 * KQ_S]);
    jvs[308 * KQ_S] = 0.0 - (r[81 * KQ_S] * v[120 * KQ_S] * v[155 * KQ_S]) + (r[248 * KQ_S] * v[119 * KQ_S]);
    jvs[309 * KQ_S] = 0.0 + (r[8 * KQ_S]);
    jvs[310 * KQ_S] = 0.0 - (r[24 * KQ_S]) - (r[82 * KQ_S] * v[155 * KQ_S] * v[156 * KQ_S]) - (r[83 * KQ_S] * v[156 * KQ_S]) - (r[103 * KQ_S]);
    jvs[311 * KQ_S] = 0.0 - (r[82 * KQ_S] * v[121 * KQ_S] * v[156 * KQ_S]);
    jvs[312 * KQ_S] = 0.0 - (r[82 * KQ_S] * v[121 * KQ_S] * v[155 * KQ_S]) - (r[83 * KQ_S] * v[121 * KQ_S]);
    jvs[313 * KQ_S] = 0.0 - (r[246 * KQ_S] * f[0 * KQ_S]) - (r[262 * KQ_S]);
    jvs[314 * KQ_S] = 0.0 + (r[240 * KQ_S] * v[153 * KQ_S]);
    jvs[315 * KQ_S] = 0.0 + 0x1.0000000000000p+1 * (r[244 * KQ_S] * 0x1.0000000000000p+1 * v[142 * KQ_S]);
    jvs[316 * KQ_S] = 0.0 + (r[240 * KQ_S] * v[126 * KQ_S]);
    jvs[317 * KQ_S] = 0.0 + (r[49 * KQ_S]);
    jvs[318 * KQ_S] = 0.0 + (r[246 * KQ_S] * f[0 * KQ_S]);
    jvs[319 * KQ_S] = 0.0 - (r[50 * KQ_S]) - (r[63 * KQ_S] * v[155 * KQ_S]) - (r[129 * KQ_S]);
    jvs[320 * KQ_S] = 0.0;
    jvs[321 * KQ_S] = 0.0;
    jvs[322 * KQ_S] = 0.0 + (r[64 * KQ_S] * v[155 * KQ_S]);
    jvs[323 * KQ_S] = 0.0 - (r[63 * KQ_S] * v[123 * KQ_S]) + (r[64 * KQ_S] * v[153 * KQ_S]);
    jvs[324 * KQ_S] = 0.0 + (r[2 * KQ_S]);
    jvs[325 * KQ_S] = 0.0 + (r[57 * KQ_S] * v[155 * KQ_S]);
}

KQ_HD KQ_NOINLINE void kqu_jac_4(const double* v, const double* f, const double* r, double* jvs)
{
    jvs[326 * KQ_S] = 0.0 - (r[18 * KQ_S]) - (r[43 * KQ_S]) - (r[97 * KQ_S]);
    jvs[327 * KQ_S] = 0.0 + 0x1.0000000000000p+1 * (r[200 * KQ_S] * v[160 * KQ_S]);
    jvs[328 * KQ_S] = 0.0 + (r[202 * KQ_S] * v[160 * KQ_S]);
    jvs[329 * KQ_S] = 0.0 + (r[201 * KQ_S] * v[160 * KQ_S]);
    jvs[330 * KQ_S] = 0.0 + (r[205 * KQ_S] * v[160 * KQ_S]);
    jvs[331 * KQ_S] = 0.0 + (r[204 * KQ_S] * v[160 * KQ_S]);
    jvs[332 * KQ_S] = 0.0 + (r[249 * KQ_S] * v[160 * KQ_S]);
    jvs[333 * KQ_S] = 0.0 + (r[209 * KQ_S] * v[160 * KQ_S]);
    jvs[334 * KQ_S] = 0.0 + (r[57 * KQ_S] * v[114 * KQ_S]);
    jvs[335 * KQ_S] = 0.0 + 0x1.0000000000000p+1 * (r[200 * KQ_S] * v[128 * KQ_S]) + (r[201 * KQ_S] * v[131 * KQ_S]) + (r[202 * KQ_S] * v[130 * KQ_S]) + (r[204 * KQ_S] * v[133 * KQ_S]) + (r[205 * KQ_S] * v[132 * KQ_S]) + (r[209 * KQ_S] * v[141 * KQ_S]) + (r[249 * KQ_S] * v[137 * KQ_S]);
    jvs[336 * KQ_S] = 0.0 + (r[14 * KQ_S]);
    jvs[337 * KQ_S] = 0.0 - (r[30 * KQ_S]) - (r[52 * KQ_S]) - (r[94 * KQ_S] * v[160 * KQ_S]) - (r[133 * KQ_S]);
    jvs[338 * KQ_S] = 0.0 + (r[66 * KQ_S] * v[155 * KQ_S]);
    jvs[339 * KQ_S] = 0.0 + (r[66 * KQ_S] * v[151 * KQ_S]);
    jvs[340 * KQ_S] = 0.0 - (r[94 * KQ_S] * v[125 * KQ_S]);
    jvs[341 * KQ_S] = 0.0 + (r[227 * KQ_S]);
    jvs[342 * KQ_S] = 0.0 - (r[229 * KQ_S]) - (r[240 * KQ_S] * v[153 * KQ_S]) - (r[241 * KQ_S] * v[156 * KQ_S]) - (r[260 * KQ_S]);
    jvs[343 * KQ_S] = 0.0 - (r[240 * KQ_S] * v[126 * KQ_S]);
    jvs[344 * KQ_S] = 0.0 - (r[241 * KQ_S] * v[126 * KQ_S]);
    jvs[345 * KQ_S] = 0.0 - (r[245 * KQ_S] * v[155 * KQ_S] * v[156 * KQ_S]) - (r[266 * KQ_S]);
    jvs[346 * KQ_S] = 0.0 + (r[243 * KQ_S] * v[154 * KQ_S]);
    jvs[347 * KQ_S] = 0.0 + (r[243 * KQ_S] * v[142 * KQ_S]);
    jvs[348 * KQ_S] = 0.0 - (r[245 * KQ_S] * v[127 * KQ_S] * v[156 * KQ_S]);
    jvs[349 * KQ_S] = 0.0 - (r[245 * KQ_S] * v[127 * KQ_S] * v[155 * KQ_S]);
    jvs[350 * KQ_S] = 0.0 - (r[177 * KQ_S]) - (r[200 * KQ_S] * v[160 * KQ_S]) - (r[213 * KQ_S]);
    jvs[351 * KQ_S] = 0.0 + (r[183 * KQ_S] * v[155 * KQ_S]);
    jvs[352 * KQ_S] = 0.0 + (r[198 * KQ_S] * v[160 * KQ_S]);
    jvs[353 * KQ_S] = 0.0 + (r[183 * KQ_S] * v[131 * KQ_S]);
    jvs[354 * KQ_S] = 0.0 + (r[198 * KQ_S] * v[136 * KQ_S]) - (r[200 * KQ_S] * v[128 * KQ_S]);
    jvs[355 * KQ_S] = 0.0 - (r[67 * KQ_S] * v[155 * KQ_S]) - (r[91 * KQ_S]) - (r[135 * KQ_S]);
    jvs[356 * KQ_S] = 0.0 + (r[53 * KQ_S]);
    jvs[357 * KQ_S] = 0.0 + (r[238 * KQ_S] * v[158 * KQ_S]);
    jvs[358 * KQ_S] = 0.0 - (r[67 * KQ_S] * v[129 * KQ_S]);
    jvs[359 * KQ_S] = 0.0 + (r[238 * KQ_S] * v[150 * KQ_S]);
    jvs[360 * KQ_S] = 0.0 - (r[184 * KQ_S] * v[155 * KQ_S]) - (r[202 * KQ_S] * v[160 * KQ_S]) - (r[215 * KQ_S]);
    jvs[361 * KQ_S] = 0.0 + (r[178 * KQ_S]);
    jvs[362 * KQ_S] = 0.0 - (r[184 * KQ_S] * v[130 * KQ_S]);
    jvs[363 * KQ_S] = 0.0 - (r[202 * KQ_S] * v[130 * KQ_S]);
    jvs[364 * KQ_S] = 0.0 + (r[177 * KQ_S]);
    jvs[365 * KQ_S] = 0.0 + (r[184 * KQ_S] * v[155 * KQ_S]);
    jvs[366 * KQ_S] = 0.0 - (r[178 * KQ_S]) - (r[183 * KQ_S] * v[155 * KQ_S]) - (r[201 * KQ_S] * v[160 * KQ_S]) - (r[214 * KQ_S]);
    jvs[367 * KQ_S] = 0.0;
    jvs[368 * KQ_S] = 0.0 + (r[199 * KQ_S] * v[160 * KQ_S]);
    jvs[369 * KQ_S] = 0.0 - (r[183 * KQ_S] * v[131 * KQ_S]) + (r[184 * KQ_S] * v[130 * KQ_S]);
    jvs[370 * KQ_S] = 0.0 + (r[199 * KQ_S] * v[140 * KQ_S]) - (r[201 * KQ_S] * v[131 * KQ_S]);
    jvs[371 * KQ_S] = 0.0 + 0x1.d70a3e0000000p-1 * (r[203 * KQ_S] * v[160 * KQ_S]);
    jvs[372 * KQ_S] = 0.0 - (r[185 * KQ_S] * v[155 * KQ_S]) - (r[205 * KQ_S] * v[160 * KQ_S]) - (r[217 * KQ_S]);
    jvs[373 * KQ_S] = 0.0 + (r[179 * KQ_S]);
    jvs[374 * KQ_S] = 0.0 - (r[185 * KQ_S] * v[132 * KQ_S]);
    jvs[375 * KQ_S] = 0.0 + 0x1.d70a3e0000000p-1 * (r[203 * KQ_S] * v[112 * KQ_S]) - (r[205 * KQ_S] * v[132 * KQ_S]);
    jvs[376 * KQ_S] = 0.0 + (r[170 * KQ_S]);
    jvs[377 * KQ_S] = 0.0 + (r[185 * KQ_S] * v[155 * KQ_S]);
    jvs[378 * KQ_S] = 0.0 - (r[175 * KQ_S]) - (r[179 * KQ_S]) - (r[204 * KQ_S] * v[160 * KQ_S]) - (r[216 * KQ_S]);
}

KQ_HD KQ_NOINLINE void kqu_jac_5(const double* v, const double* f, const double* r, double* jvs)
{
    jvs[379 * KQ_S] = 0.0 + (r[185 * KQ_S] * v[132 * KQ_S]);
    jvs[380 * KQ_S] = 0.0 - (r[204 * KQ_S] * v[133 * KQ_S]);
    jvs[381 * KQ_S] = 0.0 + (r[167 * KQ_S]);
    jvs[382 * KQ_S] = 0.0 + (r[204 * KQ_S] * v[160 * KQ_S]);
    jvs[383 * KQ_S] = 0.0 - (r[172 * KQ_S]) - (r[181 * KQ_S]) - (r[206 * KQ_S] * v[160 * KQ_S]) - (r[218 * KQ_S]);
    jvs[384 * KQ_S] = 0.0 + (r[187 * KQ_S] * v[155 * KQ_S]);
    jvs[385 * KQ_S] = 0.0 + (r[187 * KQ_S] * v[135 * KQ_S]);
    jvs[386 * KQ_S] = 0.0 + (r[204 * KQ_S] * v[133 * KQ_S]) - (r[206 * KQ_S] * v[134 * KQ_S]);
    jvs[387 * KQ_S] = 0.0 + (r[205 * KQ_S] * v[160 * KQ_S]);
    jvs[388 * KQ_S] = 0.0;
    jvs[389 * KQ_S] = 0.0 + (r[181 * KQ_S]);
    jvs[390 * KQ_S] = 0.0 - (r[187 * KQ_S] * v[155 * KQ_S]) - (r[207 * KQ_S] * v[160 * KQ_S]) - (r[219 * KQ_S]);
    jvs[391 * KQ_S] = 0.0 - (r[187 * KQ_S] * v[135 * KQ_S]);
    jvs[392 * KQ_S] = 0.0 + (r[205 * KQ_S] * v[132 * KQ_S]) - (r[207 * KQ_S] * v[135 * KQ_S]);
    jvs[393 * KQ_S] = 0.0 + (r[197 * KQ_S] * v[160 * KQ_S]);
    jvs[394 * KQ_S] = 0.0 + 0x1.b333340000000p-1 * (r[206 * KQ_S] * v[160 * KQ_S]);
    jvs[395 * KQ_S] = 0.0;
    jvs[396 * KQ_S] = 0.0 - (r[176 * KQ_S]) - (r[198 * KQ_S] * v[160 * KQ_S]) - (r[211 * KQ_S]);
    jvs[397 * KQ_S] = 0.0 + (r[182 * KQ_S] * v[155 * KQ_S]);
    jvs[398 * KQ_S] = 0.0 + (r[182 * KQ_S] * v[140 * KQ_S]);
    jvs[399 * KQ_S] = 0.0 + (r[197 * KQ_S] * v[105 * KQ_S]) - (r[198 * KQ_S] * v[136 * KQ_S]) + 0x1.b333340000000p-1 * (r[206 * KQ_S] * v[134 * KQ_S]);
    jvs[400 * KQ_S] = 0.0 - (r[60 * KQ_S] * v[155 * KQ_S]) - (r[128 * KQ_S]) - (r[249 * KQ_S] * v[160 * KQ_S]);
    jvs[401 * KQ_S] = 0.0 + (r[46 * KQ_S]);
    jvs[402 * KQ_S] = 0.0 - (r[60 * KQ_S] * v[137 * KQ_S]);
    jvs[403 * KQ_S] = 0.0 - (r[249 * KQ_S] * v[137 * KQ_S]);
    jvs[404 * KQ_S] = 0.0 + (r[193 * KQ_S] * v[160 * KQ_S]);
    jvs[405 * KQ_S] = 0.0 - (r[180 * KQ_S]) - (r[195 * KQ_S] * v[160 * KQ_S]) - (r[222 * KQ_S]);
    jvs[406 * KQ_S] = 0.0 + (r[186 * KQ_S] * v[155 * KQ_S]);
    jvs[407 * KQ_S] = 0.0 + (r[186 * KQ_S] * v[139 * KQ_S]);
    jvs[408 * KQ_S] = 0.0 + (r[193 * KQ_S] * v[104 * KQ_S]) - (r[195 * KQ_S] * v[138 * KQ_S]);
    jvs[409 * KQ_S] = 0.0 + (r[180 * KQ_S]);
    jvs[410 * KQ_S] = 0.0 - (r[186 * KQ_S] * v[155 * KQ_S]) - (r[196 * KQ_S] * v[160 * KQ_S]) - (r[223 * KQ_S]);
    jvs[411 * KQ_S] = 0.0 - (r[186 * KQ_S] * v[139 * KQ_S]);
    jvs[412 * KQ_S] = 0.0 - (r[196 * KQ_S] * v[139 * KQ_S]);
    jvs[413 * KQ_S] = 0.0 + 0x1.47ae140000000p-4 * (r[203 * KQ_S] * v[160 * KQ_S]);
    jvs[414 * KQ_S] = 0.0 + 0x1.b333340000000p-1 * (r[207 * KQ_S] * v[160 * KQ_S]);
    jvs[415 * KQ_S] = 0.0 + (r[176 * KQ_S]);
    jvs[416 * KQ_S] = 0.0 + (r[195 * KQ_S] * v[160 * KQ_S]);
    jvs[417 * KQ_S] = 0.0 + (r[196 * KQ_S] * v[160 * KQ_S]);
    jvs[418 * KQ_S] = 0.0 - (r[182 * KQ_S] * v[155 * KQ_S]) - (r[199 * KQ_S] * v[160 * KQ_S]) - (r[212 * KQ_S]);
    jvs[419 * KQ_S] = 0.0 - (r[182 * KQ_S] * v[140 * KQ_S]);
    jvs[420 * KQ_S] = 0.0 + (r[195 * KQ_S] * v[138 * KQ_S]) + (r[196 * KQ_S] * v[139 * KQ_S]) - (r[199 * KQ_S] * v[140 * KQ_S]) + 0x1.47ae140000000p-4 * (r[203 * KQ_S] * v[112 * KQ_S]) + 0x1.b333340000000p-1 * (r[207 * KQ_S] * v[135 * KQ_S]);
    jvs[421 * KQ_S] = 0.0 + (r[6 * KQ_S]);
    jvs[422 * KQ_S] = 0.0 + (r[60 * KQ_S] * v[155 * KQ_S]);
    jvs[423 * KQ_S] = 0.0 - (r[22 * KQ_S]) - (r[46 * KQ_S]) - (r[101 * KQ_S]) - (r[209 * KQ_S] * v[160 * KQ_S]);
    jvs[424 * KQ_S] = 0.0 + (r[254 * KQ_S] * v[160 * KQ_S]);
    jvs[425 * KQ_S] = 0.0 + (r[208 * KQ_S] * v[160 * KQ_S]);
    jvs[426 * KQ_S] = 0.0 + (r[60 * KQ_S] * v[137 * KQ_S]);
    jvs[427 * KQ_S] = 0.0 + (r[208 * KQ_S] * v[148 * KQ_S]) - (r[209 * KQ_S] * v[141 * KQ_S]) + (r[254 * KQ_S] * v[147 * KQ_S]);
    jvs[428 * KQ_S] = 0.0 + (r[242 * KQ_S] * f[2 * KQ_S]);
    jvs[429 * KQ_S] = 0.0;
    jvs[430 * KQ_S] = 0.0;
    jvs[431 * KQ_S] = 0.0 - (r[243 * KQ_S] * v[154 * KQ_S]) + -0x1.0000000000000p+1 * (r[244 * KQ_S] * 0x1.0000000000000p+1 * v[142 * KQ_S]) - (r[265 * KQ_S]);
    jvs[432 * KQ_S] = 0.0;
    jvs[433 * KQ_S] = 0.0 - (r[243 * KQ_S] * v[142 * KQ_S]);
    jvs[434 * KQ_S] = 0.0;
    jvs[435 * KQ_S] = 0.0;
    jvs[436 * KQ_S] = 0.0 + (r[168 * KQ_S]);
}

KQ_HD KQ_NOINLINE void kqu_jac_6(const double* v, const double* f, const double* r, double* jvs)
{
    jvs[437 * KQ_S] = 0.0 + 0x1.0000000000000p+1 * (r[247 * KQ_S] * 0x1.0000000000000p+1 * v[119 * KQ_S]);
    jvs[438 * KQ_S] = 0.0 - (r[173 * KQ_S]) - (r[188 * KQ_S] * f[0 * KQ_S]) - (r[224 * KQ_S]) - (r[250 * KQ_S] * v[156 * KQ_S]) - (r[251 * KQ_S] * v[159 * KQ_S]);
    jvs[439 * KQ_S] = 0.0 + (r[252 * KQ_S]);
    jvs[440 * KQ_S] = 0.0 + (r[189 * KQ_S]);
    jvs[441 * KQ_S] = 0.0 - (r[250 * KQ_S] * v[143 * KQ_S]);
    jvs[442 * KQ_S] = 0.0 - (r[251 * KQ_S] * v[143 * KQ_S]);
    jvs[443 * KQ_S] = 0.0 - (r[75 * KQ_S] * v[144 * KQ_S]) - (r[78 * KQ_S] * v[13 * KQ_S] * v[144 * KQ_S]);
    jvs[444 * KQ_S] = 0.0 - (r[72 * KQ_S] * v[144 * KQ_S]) - (r[78 * KQ_S] * v[12 * KQ_S] * v[144 * KQ_S]);
    jvs[445 * KQ_S] = 0.0 + (r[0 * KQ_S]);
    jvs[446 * KQ_S] = 0.0 - (r[16 * KQ_S]) - (r[40 * KQ_S]) - (r[69 * KQ_S] * v[157 * KQ_S]) - (r[72 * KQ_S] * v[13 * KQ_S]) - (r[75 * KQ_S] * v[12 * KQ_S]) - (r[78 * KQ_S] * v[12 * KQ_S] * v[13 * KQ_S]) - (r[87 * KQ_S] * v[158 * KQ_S]) - (r[95 * KQ_S]);
    jvs[447 * KQ_S] = 0.0 + (r[54 * KQ_S] * v[156 * KQ_S]);
    jvs[448 * KQ_S] = 0.0 + (r[54 * KQ_S] * v[155 * KQ_S]);
    jvs[449 * KQ_S] = 0.0 - (r[69 * KQ_S] * v[144 * KQ_S]);
    jvs[450 * KQ_S] = 0.0 - (r[87 * KQ_S] * v[144 * KQ_S]);
    jvs[451 * KQ_S] = 0.0 + (r[4 * KQ_S]);
    jvs[452 * KQ_S] = 0.0 - (r[20 * KQ_S]) - (r[68 * KQ_S] * v[155 * KQ_S] * v[156 * KQ_S]) - (r[99 * KQ_S]) - (r[192 * KQ_S]) - (r[235 * KQ_S] * v[160 * KQ_S]);
    jvs[453 * KQ_S] = 0.0 + (r[85 * KQ_S] * v[154 * KQ_S]);
    jvs[454 * KQ_S] = 0.0 + (r[84 * KQ_S] * 0x1.0000000000000p+1 * v[154 * KQ_S]) + (r[85 * KQ_S] * v[150 * KQ_S]);
    jvs[455 * KQ_S] = 0.0 - (r[68 * KQ_S] * v[145 * KQ_S] * v[156 * KQ_S]);
    jvs[456 * KQ_S] = 0.0 - (r[68 * KQ_S] * v[145 * KQ_S] * v[155 * KQ_S]);
    jvs[457 * KQ_S] = 0.0 + (r[232 * KQ_S] * 0x1.0000000000000p+1 * v[160 * KQ_S]) - (r[235 * KQ_S] * v[145 * KQ_S]);
    jvs[458 * KQ_S] = 0.0 + (r[32 * KQ_S]);
    jvs[459 * KQ_S] = 0.0 + (r[42 * KQ_S]);
    jvs[460 * KQ_S] = 0.0 - (r[152 * KQ_S] * v[146 * KQ_S]);
    jvs[461 * KQ_S] = 0.0 + (r[240 * KQ_S] * v[153 * KQ_S]) + (r[241 * KQ_S] * v[156 * KQ_S]);
    jvs[462 * KQ_S] = 0.0 - (r[56 * KQ_S] * v[155 * KQ_S]) - (r[109 * KQ_S]) - (r[152 * KQ_S] * v[115 * KQ_S]) - (r[231 * KQ_S]);
    jvs[463 * KQ_S] = 0.0 + (r[90 * KQ_S] * v[156 * KQ_S]);
    jvs[464 * KQ_S] = 0.0 + (r[92 * KQ_S] * v[157 * KQ_S]);
    jvs[465 * KQ_S] = 0.0 + (r[240 * KQ_S] * v[126 * KQ_S]);
    jvs[466 * KQ_S] = 0.0 - (r[56 * KQ_S] * v[146 * KQ_S]);
    jvs[467 * KQ_S] = 0.0 + (r[90 * KQ_S] * v[149 * KQ_S]) + (r[241 * KQ_S] * v[126 * KQ_S]);
    jvs[468 * KQ_S] = 0.0 + (r[92 * KQ_S] * v[151 * KQ_S]);
    jvs[469 * KQ_S] = 0.0 + (r[250 * KQ_S] * v[156 * KQ_S]) + (r[251 * KQ_S] * v[159 * KQ_S]);
    jvs[470 * KQ_S] = 0.0 - (r[252 * KQ_S]) - (r[253 * KQ_S] * v[152 * KQ_S]) - (r[254 * KQ_S] * v[160 * KQ_S]) - (r[264 * KQ_S]);
    jvs[471 * KQ_S] = 0.0;
    jvs[472 * KQ_S] = 0.0 - (r[253 * KQ_S] * v[147 * KQ_S]);
    jvs[473 * KQ_S] = 0.0 + (r[250 * KQ_S] * v[143 * KQ_S]);
    jvs[474 * KQ_S] = 0.0 + (r[251 * KQ_S] * v[143 * KQ_S]);
    jvs[475 * KQ_S] = 0.0 - (r[254 * KQ_S] * v[147 * KQ_S]);
    jvs[476 * KQ_S] = 0.0 + 0x1.3333340000000p-3 * (r[206 * KQ_S] * v[160 * KQ_S]);
    jvs[477 * KQ_S] = 0.0 + 0x1.3333340000000p-3 * (r[207 * KQ_S] * v[160 * KQ_S]);
    jvs[478 * KQ_S] = 0.0 + (r[188 * KQ_S] * f[0 * KQ_S]);
    jvs[479 * KQ_S] = 0.0 + (r[253 * KQ_S] * v[152 * KQ_S]);
    jvs[480 * KQ_S] = 0.0 - (r[189 * KQ_S]) - (r[208 * KQ_S] * v[160 * KQ_S]) - (r[220 * KQ_S]);
    jvs[481 * KQ_S] = 0.0 + (r[253 * KQ_S] * v[147 * KQ_S]);
    jvs[482 * KQ_S] = 0.0;
    jvs[483 * KQ_S] = 0.0;
    jvs[484 * KQ_S] = 0.0;
    jvs[485 * KQ_S] = 0.0 + 0x1.3333340000000p-3 * (r[206 * KQ_S] * v[134 * KQ_S]) + 0x1.3333340000000p-3 * (r[207 * KQ_S] * v[135 * KQ_S]) - (r[208 * KQ_S] * v[148 * KQ_S]);
    jvs[486 * KQ_S] = 0.0 + (r[15 * KQ_S]);
    jvs[487 * KQ_S] = 0.0 + (r[67 * KQ_S] * v[155 * KQ_S]);
}

KQ_HD KQ_NOINLINE void kqu_jac_7(const double* v, const double* f, const double* r, double* jvs)
{
    jvs[488 * KQ_S] = 0.0 - (r[31 * KQ_S]) - (r[53 * KQ_S]) - (r[90 * KQ_S] * v[156 * KQ_S]) - (r[136 * KQ_S]) - (r[239 * KQ_S]);
    jvs[489 * KQ_S] = 0.0;
    jvs[490 * KQ_S] = 0.0 + (r[237 * KQ_S] * v[158 * KQ_S]);
    jvs[491 * KQ_S] = 0.0 + (r[67 * KQ_S] * v[129 * KQ_S]);
    jvs[492 * KQ_S] = 0.0 - (r[90 * KQ_S] * v[149 * KQ_S]);
    jvs[493 * KQ_S] = 0.0 + (r[237 * KQ_S] * v[154 * KQ_S]);
    jvs[494 * KQ_S] = 0.0 - (r[65 * KQ_S] * v[155 * KQ_S]) - (r[85 * KQ_S] * v[154 * KQ_S]) - (r[86 * KQ_S] * v[157 * KQ_S]) - (r[130 * KQ_S]) - (r[234 * KQ_S] * v[160 * KQ_S]) - (r[238 * KQ_S] * v[158 * KQ_S]);
    jvs[495 * KQ_S] = 0.0 + (r[51 * KQ_S]) - (r[85 * KQ_S] * v[150 * KQ_S]);
    jvs[496 * KQ_S] = 0.0 - (r[65 * KQ_S] * v[150 * KQ_S]);
    jvs[497 * KQ_S] = 0.0 - (r[86 * KQ_S] * v[150 * KQ_S]);
    jvs[498 * KQ_S] = 0.0 - (r[238 * KQ_S] * v[150 * KQ_S]);
    jvs[499 * KQ_S] = 0.0 - (r[234 * KQ_S] * v[150 * KQ_S]);
    jvs[500 * KQ_S] = 0.0 + (r[52 * KQ_S]);
    jvs[501 * KQ_S] = 0.0 + (r[91 * KQ_S]);
    jvs[502 * KQ_S] = 0.0 + 0x1.0000000000000p+1 * (r[87 * KQ_S] * v[158 * KQ_S]);
    jvs[503 * KQ_S] = 0.0;
    jvs[504 * KQ_S] = 0.0;
    jvs[505 * KQ_S] = 0.0 - (r[66 * KQ_S] * v[155 * KQ_S]) - (r[92 * KQ_S] * v[157 * KQ_S]) - (r[93 * KQ_S] * v[160 * KQ_S]) - (r[134 * KQ_S]);
    jvs[506 * KQ_S] = 0.0;
    jvs[507 * KQ_S] = 0.0 - (r[66 * KQ_S] * v[151 * KQ_S]);
    jvs[508 * KQ_S] = 0.0 + 0x1.0000000000000p+1 * (r[88 * KQ_S] * v[158 * KQ_S]);
    jvs[509 * KQ_S] = 0.0 - (r[92 * KQ_S] * v[151 * KQ_S]);
    jvs[510 * KQ_S] = 0.0 + 0x1.0000000000000p+1 * (r[87 * KQ_S] * v[144 * KQ_S]) + 0x1.0000000000000p+1 * (r[88 * KQ_S] * v[156 * KQ_S]) + 0x1.0000000000000p+1 * (r[89 * KQ_S] * v[159 * KQ_S]);
    jvs[511 * KQ_S] = 0.0 + 0x1.0000000000000p+1 * (r[89 * KQ_S] * v[158 * KQ_S]);
    jvs[512 * KQ_S] = 0.0 - (r[93 * KQ_S] * v[151 * KQ_S]);
    jvs[513 * KQ_S] = 0.0 + (r[45 * KQ_S]);
    jvs[514 * KQ_S] = 0.0 - (r[59 * KQ_S] * v[152 * KQ_S]);
    jvs[515 * KQ_S] = 0.0 + (r[202 * KQ_S] * v[160 * KQ_S]);
    jvs[516 * KQ_S] = 0.0;
    jvs[517 * KQ_S] = 0.0;
    jvs[518 * KQ_S] = 0.0 + (r[249 * KQ_S] * v[160 * KQ_S]);
    jvs[519 * KQ_S] = 0.0;
    jvs[520 * KQ_S] = 0.0;
    jvs[521 * KQ_S] = 0.0 + (r[251 * KQ_S] * v[159 * KQ_S]);
    jvs[522 * KQ_S] = 0.0 + (r[231 * KQ_S]);
    jvs[523 * KQ_S] = 0.0 - (r[253 * KQ_S] * v[152 * KQ_S]);
    jvs[524 * KQ_S] = 0.0;
    jvs[525 * KQ_S] = 0.0;
    jvs[526 * KQ_S] = 0.0 + (r[85 * KQ_S] * v[154 * KQ_S]) + (r[86 * KQ_S] * v[157 * KQ_S]) + (r[234 * KQ_S] * v[160 * KQ_S]);
    jvs[527 * KQ_S] = 0.0 + (r[93 * KQ_S] * v[160 * KQ_S]);
    jvs[528 * KQ_S] = 0.0 - (r[59 * KQ_S] * v[108 * KQ_S]) - (r[62 * KQ_S] * v[155 * KQ_S]) - (r[123 * KQ_S]) - (r[253 * KQ_S] * v[147 * KQ_S]);
    jvs[529 * KQ_S] = 0.0;
    jvs[530 * KQ_S] = 0.0 + (r[85 * KQ_S] * v[150 * KQ_S]);
    jvs[531 * KQ_S] = 0.0 - (r[62 * KQ_S] * v[152 * KQ_S]);
    jvs[532 * KQ_S] = 0.0;
    jvs[533 * KQ_S] = 0.0 + (r[86 * KQ_S] * v[150 * KQ_S]);
    jvs[534 * KQ_S] = 0.0;
    jvs[535 * KQ_S] = 0.0 + (r[251 * KQ_S] * v[143 * KQ_S]);
    jvs[536 * KQ_S] = 0.0 + (r[93 * KQ_S] * v[151 * KQ_S]) + (r[202 * KQ_S] * v[130 * KQ_S]) + (r[234 * KQ_S] * v[150 * KQ_S]) + (r[249 * KQ_S] * v[137 * KQ_S]);
    jvs[537 * KQ_S] = 0.0 + (r[36 * KQ_S]);
    jvs[538 * KQ_S] = 0.0 + (r[75 * KQ_S] * v[144 * KQ_S]) + (r[76 * KQ_S] * v[156 * KQ_S]) + (r[77 * KQ_S] * v[159 * KQ_S]) + (r[78 * KQ_S] * v[13 * KQ_S] * v[144 * KQ_S]) + (r[79 * KQ_S] * v[13 * KQ_S] * v[156 * KQ_S]) + (r[80 * KQ_S] * v[13 * KQ_S] * v[159 * KQ_S]);
    jvs[539 * KQ_S] = 0.0 + (r[72 * KQ_S] * v[144 * KQ_S]) + (r[73 * KQ_S] * v[156 * KQ_S]) + (r[74 * KQ_S] * v[159 * KQ_S]) + (r[78 * KQ_S] * v[12 * KQ_S] * v[144 * KQ_S]) + (r[79 * KQ_S] * v[12 * KQ_S] * v[156 * KQ_S]) + (r[80 * KQ_S] * v[12 * KQ_S] * v[159 * KQ_S]);
    jvs[540 * KQ_S] = 0.0 - (r[154 * KQ_S] * v[153 * KQ_S]);
    jvs[541 * KQ_S] = 0.0 - (r[156 * KQ_S] * v[153 * KQ_S]);
    jvs[542 * KQ_S] = 0.0 - (r[147 * KQ_S] * v[153 * KQ_S]) - (r[151 * KQ_S] * v[153 * KQ_S]);
}

KQ_HD KQ_NOINLINE void kqu_jac_8(const double* v, const double* f, const double* r, double* jvs)
{
    jvs[543 * KQ_S] = 0.0 + (r[81 * KQ_S] * v[155 * KQ_S] * v[156 * KQ_S]);
    jvs[544 * KQ_S] = 0.0 + (r[82 * KQ_S] * v[155 * KQ_S] * v[156 * KQ_S]) + (r[83 * KQ_S] * v[156 * KQ_S]);
    jvs[545 * KQ_S] = 0.0 + (r[50 * KQ_S]);
    jvs[546 * KQ_S] = 0.0 - (r[240 * KQ_S] * v[153 * KQ_S]);
    jvs[547 * KQ_S] = 0.0 + 0x1.0000000000000p+1 * (r[245 * KQ_S] * v[155 * KQ_S] * v[156 * KQ_S]);
    jvs[548 * KQ_S] = 0.0;
    jvs[549 * KQ_S] = 0.0 + (r[69 * KQ_S] * v[157 * KQ_S]) + (r[72 * KQ_S] * v[13 * KQ_S]) + (r[75 * KQ_S] * v[12 * KQ_S]) + (r[78 * KQ_S] * v[12 * KQ_S] * v[13 * KQ_S]) + (r[87 * KQ_S] * v[158 * KQ_S]);
    jvs[550 * KQ_S] = 0.0 + (r[68 * KQ_S] * v[155 * KQ_S] * v[156 * KQ_S]);
    jvs[551 * KQ_S] = 0.0;
    jvs[552 * KQ_S] = 0.0 + (r[90 * KQ_S] * v[156 * KQ_S]);
    jvs[553 * KQ_S] = 0.0;
    jvs[554 * KQ_S] = 0.0;
    jvs[555 * KQ_S] = 0.0 - (r[64 * KQ_S] * v[155 * KQ_S]) - (r[108 * KQ_S]) - (r[147 * KQ_S] * v[115 * KQ_S]) - (r[151 * KQ_S] * v[115 * KQ_S]) - (r[154 * KQ_S] * v[75 * KQ_S]) - (r[156 * KQ_S] * v[77 * KQ_S]) - (r[240 * KQ_S] * v[126 * KQ_S]);
    jvs[556 * KQ_S] = 0.0;
    jvs[557 * KQ_S] = 0.0 - (r[64 * KQ_S] * v[153 * KQ_S]) + (r[68 * KQ_S] * v[145 * KQ_S] * v[156 * KQ_S]) + (r[81 * KQ_S] * v[120 * KQ_S] * v[156 * KQ_S]) + (r[82 * KQ_S] * v[121 * KQ_S] * v[156 * KQ_S]) + 0x1.0000000000000p+1 * (r[245 * KQ_S] * v[127 * KQ_S] * v[156 * KQ_S]);
    jvs[558 * KQ_S] = 0.0 + (r[68 * KQ_S] * v[145 * KQ_S] * v[155 * KQ_S]) + (r[70 * KQ_S] * v[157 * KQ_S]) + (r[73 * KQ_S] * v[13 * KQ_S]) + (r[76 * KQ_S] * v[12 * KQ_S]) + (r[79 * KQ_S] * v[12 * KQ_S] * v[13 * KQ_S]) + (r[81 * KQ_S] * v[120 * KQ_S] * v[155 * KQ_S]) + (r[82 * KQ_S] * v[121 * KQ_S] * v[155 * KQ_S]) + (r[83 * KQ_S] * v[121 * KQ_S]) + (r[88 * KQ_S] * v[158 * KQ_S]) + (r[90 * KQ_S] * v[149 * KQ_S]) + 0x1.0000000000000p+1 * (r[245 * KQ_S] * v[127 * KQ_S] * v[155 * KQ_S]);
    jvs[559 * KQ_S] = 0.0 + (r[69 * KQ_S] * v[144 * KQ_S]) + (r[70 * KQ_S] * v[156 * KQ_S]) + (r[71 * KQ_S] * v[159 * KQ_S]);
    jvs[560 * KQ_S] = 0.0 + (r[87 * KQ_S] * v[144 * KQ_S]) + (r[88 * KQ_S] * v[156 * KQ_S]) + (r[89 * KQ_S] * v[159 * KQ_S]);
    jvs[561 * KQ_S] = 0.0 + (r[71 * KQ_S] * v[157 * KQ_S]) + (r[74 * KQ_S] * v[13 * KQ_S]) + (r[77 * KQ_S] * v[12 * KQ_S]) + (r[80 * KQ_S] * v[12 * KQ_S] * v[13 * KQ_S]) + (r[89 * KQ_S] * v[158 * KQ_S]);
    jvs[562 * KQ_S] = 0.0;
    jvs[563 * KQ_S] = 0.0 + (r[12 * KQ_S]);
    jvs[564 * KQ_S] = 0.0 + (r[193 * KQ_S] * v[160 * KQ_S]) + (r[194 * KQ_S] * v[160 * KQ_S]);
    jvs[565 * KQ_S] = 0.0 + (r[197 * KQ_S] * v[160 * KQ_S]);
    jvs[566 * KQ_S] = 0.0 + (r[203 * KQ_S] * v[160 * KQ_S]);
    jvs[567 * KQ_S] = 0.0 + 0x1.0000000000000p+1 * (r[247 * KQ_S] * 0x1.0000000000000p+1 * v[119 * KQ_S]);
    jvs[568 * KQ_S] = 0.0 + (r[205 * KQ_S] * v[160 * KQ_S]);
    jvs[569 * KQ_S] = 0.0 + (r[204 * KQ_S] * v[160 * KQ_S]);
    jvs[570 * KQ_S] = 0.0 + (r[198 * KQ_S] * v[160 * KQ_S]);
    jvs[571 * KQ_S] = 0.0 + (r[249 * KQ_S] * v[160 * KQ_S]);
    jvs[572 * KQ_S] = 0.0 + (r[195 * KQ_S] * v[160 * KQ_S]);
    jvs[573 * KQ_S] = 0.0 + (r[196 * KQ_S] * v[160 * KQ_S]);
    jvs[574 * KQ_S] = 0.0 + (r[199 * KQ_S] * v[160 * KQ_S]);
    jvs[575 * KQ_S] = 0.0 + (r[209 * KQ_S] * v[160 * KQ_S]);
    jvs[576 * KQ_S] = 0.0 - (r[243 * KQ_S] * v[154 * KQ_S]);
    jvs[577 * KQ_S] = 0.0 + (r[235 * KQ_S] * v[160 * KQ_S]);
    jvs[578 * KQ_S] = 0.0 + (r[254 * KQ_S] * v[160 * KQ_S]);
    jvs[579 * KQ_S] = 0.0 + (r[208 * KQ_S] * v[160 * KQ_S]);
    jvs[580 * KQ_S] = 0.0 + (r[239 * KQ_S]);
    jvs[581 * KQ_S] = 0.0 + (r[65 * KQ_S] * v[155 * KQ_S]) - (r[85 * KQ_S] * v[154 * KQ_S]);
    jvs[582 * KQ_S] = 0.0;
    jvs[583 * KQ_S] = 0.0;
}

KQ_HD KQ_NOINLINE void kqu_jac_9(const double* v, const double* f, const double* r, double* jvs)
{
    jvs[584 * KQ_S] = 0.0 - (r[28 * KQ_S]) - (r[51 * KQ_S]) + -0x1.0000000000000p+1 * (r[84 * KQ_S] * 0x1.0000000000000p+1 * v[154 * KQ_S]) - (r[85 * KQ_S] * v[150 * KQ_S]) - (r[131 * KQ_S]) - (r[233 * KQ_S] * v[160 * KQ_S]) - (r[237 * KQ_S] * v[158 * KQ_S]) - (r[243 * KQ_S] * v[142 * KQ_S]);
    jvs[585 * KQ_S] = 0.0 + (r[65 * KQ_S] * v[150 * KQ_S]);
    jvs[586 * KQ_S] = 0.0;
    jvs[587 * KQ_S] = 0.0;
    jvs[588 * KQ_S] = 0.0 - (r[237 * KQ_S] * v[154 * KQ_S]);
    jvs[589 * KQ_S] = 0.0;
    jvs[590 * KQ_S] = 0.0 + (r[193 * KQ_S] * v[104 * KQ_S]) + (r[194 * KQ_S] * v[104 * KQ_S]) + (r[195 * KQ_S] * v[138 * KQ_S]) + (r[196 * KQ_S] * v[139 * KQ_S]) + (r[197 * KQ_S] * v[105 * KQ_S]) + (r[198 * KQ_S] * v[136 * KQ_S]) + (r[199 * KQ_S] * v[140 * KQ_S]) + (r[203 * KQ_S] * v[112 * KQ_S]) + (r[204 * KQ_S] * v[133 * KQ_S]) + (r[205 * KQ_S] * v[132 * KQ_S]) + (r[208 * KQ_S] * v[148 * KQ_S]) + (r[209 * KQ_S] * v[141 * KQ_S]) - (r[233 * KQ_S] * v[154 * KQ_S]) + (r[235 * KQ_S] * v[145 * KQ_S]) + (r[249 * KQ_S] * v[137 * KQ_S]) + (r[254 * KQ_S] * v[147 * KQ_S]);
    jvs[591 * KQ_S] = 0.0 + 0x1.0000000000000p+1 * (r[75 * KQ_S] * v[144 * KQ_S]) + (r[76 * KQ_S] * v[156 * KQ_S]) + 0x1.0000000000000p+1 * (r[78 * KQ_S] * v[13 * KQ_S] * v[144 * KQ_S]) + (r[79 * KQ_S] * v[13 * KQ_S] * v[156 * KQ_S]);
    jvs[592 * KQ_S] = 0.0 + 0x1.0000000000000p+1 * (r[72 * KQ_S] * v[144 * KQ_S]) + (r[73 * KQ_S] * v[156 * KQ_S]) + 0x1.0000000000000p+1 * (r[78 * KQ_S] * v[12 * KQ_S] * v[144 * KQ_S]) + (r[79 * KQ_S] * v[12 * KQ_S] * v[156 * KQ_S]);
    jvs[593 * KQ_S] = 0.0 + (r[42 * KQ_S]);
    jvs[594 * KQ_S] = 0.0 + (r[49 * KQ_S]);
    jvs[595 * KQ_S] = 0.0 + (r[47 * KQ_S]);
    jvs[596 * KQ_S] = 0.0 - (r[61 * KQ_S] * v[155 * KQ_S]);
    jvs[597 * KQ_S] = 0.0 - (r[58 * KQ_S] * v[155 * KQ_S]);
    jvs[598 * KQ_S] = 0.0 + (r[44 * KQ_S]) - (r[57 * KQ_S] * v[155 * KQ_S]);
    jvs[599 * KQ_S] = 0.0 + (r[81 * KQ_S] * v[155 * KQ_S] * v[156 * KQ_S]);
    jvs[600 * KQ_S] = 0.0 + (r[82 * KQ_S] * v[155 * KQ_S] * v[156 * KQ_S]) + (r[83 * KQ_S] * v[156 * KQ_S]);
    jvs[601 * KQ_S] = 0.0 + (r[50 * KQ_S]) - (r[63 * KQ_S] * v[155 * KQ_S]);
    jvs[602 * KQ_S] = 0.0 + (r[43 * KQ_S]);
    jvs[603 * KQ_S] = 0.0 + (r[52 * KQ_S]);
    jvs[604 * KQ_S] = 0.0 + (r[241 * KQ_S] * v[156 * KQ_S]);
    jvs[605 * KQ_S] = 0.0 + 0x1.0000000000000p+1 * (r[245 * KQ_S] * v[155 * KQ_S] * v[156 * KQ_S]);
    jvs[606 * KQ_S] = 0.0 + (r[177 * KQ_S]);
    jvs[607 * KQ_S] = 0.0 - (r[67 * KQ_S] * v[155 * KQ_S]);
    jvs[608 * KQ_S] = 0.0 - (r[184 * KQ_S] * v[155 * KQ_S]);
    jvs[609 * KQ_S] = 0.0 + (r[178 * KQ_S]) - (r[183 * KQ_S] * v[155 * KQ_S]);
    jvs[610 * KQ_S] = 0.0 - (r[185 * KQ_S] * v[155 * KQ_S]);
    jvs[611 * KQ_S] = 0.0 + (r[179 * KQ_S]);
    jvs[612 * KQ_S] = 0.0 + (r[181 * KQ_S]);
    jvs[613 * KQ_S] = 0.0 - (r[187 * KQ_S] * v[155 * KQ_S]);
    jvs[614 * KQ_S] = 0.0 + (r[176 * KQ_S]);
    jvs[615 * KQ_S] = 0.0 - (r[60 * KQ_S] * v[155 * KQ_S]);
    jvs[616 * KQ_S] = 0.0 + (r[180 * KQ_S]) + (r[195 * KQ_S] * v[160 * KQ_S]);
    jvs[617 * KQ_S] = 0.0 - (r[186 * KQ_S] * v[155 * KQ_S]);
    jvs[618 * KQ_S] = 0.0 - (r[182 * KQ_S] * v[155 * KQ_S]);
    jvs[619 * KQ_S] = 0.0 + (r[46 * KQ_S]);
    jvs[620 * KQ_S] = 0.0;
    jvs[621 * KQ_S] = 0.0 + (r[40 * KQ_S]) + 0x1.0000000000000p+1 * (r[69 * KQ_S] * v[157 * KQ_S]) + 0x1.0000000000000p+1 * (r[72 * KQ_S] * v[13 * KQ_S]) + 0x1.0000000000000p+1 * (r[75 * KQ_S] * v[12 * KQ_S]) + 0x1.0000000000000p+1 * (r[78 * KQ_S] * v[12 * KQ_S] * v[13 * KQ_S]) + 0x1.0000000000000p+2 * (r[87 * KQ_S] * v[158 * KQ_S]);
    jvs[622 * KQ_S] = 0.0 + (r[68 * KQ_S] * v[155 * KQ_S] * v[156 * KQ_S]);
    jvs[623 * KQ_S] = 0.0 - (r[56 * KQ_S] * v[155 * KQ_S]);
    jvs[624 * KQ_S] = 0.0;
    jvs[625 * KQ_S] = 0.0;
    jvs[626 * KQ_S] = 0.0 + (r[53 * KQ_S]) + 0x1.0000000000000p+1 * (r[90 * KQ_S] * v[156 * KQ_S]);
    jvs[627 * KQ_S] = 0.0 - (r[65 * KQ_S] * v[155 * KQ_S]);
    jvs[628 * KQ_S] = 0.0 - (r[66 * KQ_S] * v[155 * KQ_S]);
    jvs[629 * KQ_S] = 0.0 - (r[62 * KQ_S] * v[155 * KQ_S]);
    jvs[630 * KQ_S] = 0.0 - (r[64 * KQ_S] * v[155 * KQ_S]);
    jvs[631 * KQ_S] = 0.0 + (r[51 * KQ_S]);
}

KQ_HD KQ_NOINLINE void kqu_jac_10(const double* v, const double* f, const double* r, double* jvs)
{
    jvs[632 * KQ_S] = 0.0 - (r[54 * KQ_S] * v[156 * KQ_S]) - (r[55 * KQ_S] * v[159 * KQ_S]) - (r[56 * KQ_S] * v[146 * KQ_S]) - (r[57 * KQ_S] * v[114 * KQ_S]) - (r[58 * KQ_S] * v[113 * KQ_S]) - (r[60 * KQ_S] * v[137 * KQ_S]) - (r[61 * KQ_S] * v[111 * KQ_S]) - (r[62 * KQ_S] * v[152 * KQ_S]) - (r[63 * KQ_S] * v[123 * KQ_S]) - (r[64 * KQ_S] * v[153 * KQ_S]) - (r[65 * KQ_S] * v[150 * KQ_S]) - (r[66 * KQ_S] * v[151 * KQ_S]) - (r[67 * KQ_S] * v[129 * KQ_S]) + (r[68 * KQ_S] * v[145 * KQ_S] * v[156 * KQ_S]) + (r[81 * KQ_S] * v[120 * KQ_S] * v[156 * KQ_S]) + (r[82 * KQ_S] * v[121 * KQ_S] * v[156 * KQ_S]) - (r[122 * KQ_S]) - (r[182 * KQ_S] * v[140 * KQ_S]) - (r[183 * KQ_S] * v[131 * KQ_S]) - (r[184 * KQ_S] * v[130 * KQ_S]) - (r[185 * KQ_S] * v[132 * KQ_S]) - (r[186 * KQ_S] * v[139 * KQ_S]) - (r[187 * KQ_S] * v[135 * KQ_S]) + 0x1.0000000000000p+1 * (r[245 * KQ_S] * v[127 * KQ_S] * v[156 * KQ_S]);
    jvs[633 * KQ_S] = 0.0 + (r[41 * KQ_S]) - (r[54 * KQ_S] * v[155 * KQ_S]) + (r[68 * KQ_S] * v[145 * KQ_S] * v[155 * KQ_S]) + (r[70 * KQ_S] * v[157 * KQ_S]) + (r[73 * KQ_S] * v[13 * KQ_S]) + (r[76 * KQ_S] * v[12 * KQ_S]) + (r[79 * KQ_S] * v[12 * KQ_S] * v[13 * KQ_S]) + (r[81 * KQ_S] * v[120 * KQ_S] * v[155 * KQ_S]) + (r[82 * KQ_S] * v[121 * KQ_S] * v[155 * KQ_S]) + (r[83 * KQ_S] * v[121 * KQ_S]) + 0x1.8000000000000p+1 * (r[88 * KQ_S] * v[158 * KQ_S]) + 0x1.0000000000000p+1 * (r[90 * KQ_S] * v[149 * KQ_S]) + (r[241 * KQ_S] * v[126 * KQ_S]) + 0x1.0000000000000p+1 * (r[245 * KQ_S] * v[127 * KQ_S] * v[155 * KQ_S]);
    jvs[634 * KQ_S] = 0.0 + 0x1.0000000000000p+1 * (r[69 * KQ_S] * v[144 * KQ_S]) + (r[70 * KQ_S] * v[156 * KQ_S]);
    jvs[635 * KQ_S] = 0.0 + 0x1.0000000000000p+2 * (r[87 * KQ_S] * v[144 * KQ_S]) + 0x1.8000000000000p+1 * (r[88 * KQ_S] * v[156 * KQ_S]) + 0x1.0000000000000p+1 * (r[89 * KQ_S] * v[159 * KQ_S]);
    jvs[636 * KQ_S] = 0.0 - (r[55 * KQ_S] * v[155 * KQ_S]) + 0x1.0000000000000p+1 * (r[89 * KQ_S] * v[158 * KQ_S]);
    jvs[637 * KQ_S] = 0.0 + (r[195 * KQ_S] * v[138 * KQ_S]);
    jvs[638 * KQ_S] = 0.0 - (r[76 * KQ_S] * v[156 * KQ_S]) - (r[79 * KQ_S] * v[13 * KQ_S] * v[156 * KQ_S]);
    jvs[639 * KQ_S] = 0.0 - (r[73 * KQ_S] * v[156 * KQ_S]) - (r[79 * KQ_S] * v[12 * KQ_S] * v[156 * KQ_S]);
    jvs[640 * KQ_S] = 0.0 - (r[248 * KQ_S] * v[156 * KQ_S]);
    jvs[641 * KQ_S] = 0.0 - (r[81 * KQ_S] * v[155 * KQ_S] * v[156 * KQ_S]);
    jvs[642 * KQ_S] = 0.0 - (r[82 * KQ_S] * v[155 * KQ_S] * v[156 * KQ_S]) - (r[83 * KQ_S] * v[156 * KQ_S]);
    jvs[643 * KQ_S] = 0.0 - (r[241 * KQ_S] * v[156 * KQ_S]);
    jvs[644 * KQ_S] = 0.0 - (r[245 * KQ_S] * v[155 * KQ_S] * v[156 * KQ_S]);
    jvs[645 * KQ_S] = 0.0;
    jvs[646 * KQ_S] = 0.0 - (r[250 * KQ_S] * v[156 * KQ_S]);
    jvs[647 * KQ_S] = 0.0 + (r[40 * KQ_S]);
    jvs[648 * KQ_S] = 0.0 - (r[68 * KQ_S] * v[155 * KQ_S] * v[156 * KQ_S]);
    jvs[649 * KQ_S] = 0.0 + (r[252 * KQ_S]) + (r[254 * KQ_S] * v[160 * KQ_S]);
    jvs[650 * KQ_S] = 0.0;
    jvs[651 * KQ_S] = 0.0 - (r[90 * KQ_S] * v[156 * KQ_S]);
    jvs[652 * KQ_S] = 0.0;
    jvs[653 * KQ_S] = 0.0;
    jvs[654 * KQ_S] = 0.0;
    jvs[655 * KQ_S] = 0.0;
    jvs[656 * KQ_S] = 0.0 - (r[54 * KQ_S] * v[156 * KQ_S]) + (r[55 * KQ_S] * v[159 * KQ_S]) - (r[68 * KQ_S] * v[145 * KQ_S] * v[156 * KQ_S]) - (r[81 * KQ_S] * v[120 * KQ_S] * v[156 * KQ_S]) - (r[82 * KQ_S] * v[121 * KQ_S] * v[156 * KQ_S]) - (r[245 * KQ_S] * v[127 * KQ_S] * v[156 * KQ_S]);
}

KQ_HD KQ_NOINLINE void kqu_jac_11(const double* v, const double* f, const double* r, double* jvs)
{
    jvs[657 * KQ_S] = 0.0 - (r[41 * KQ_S]) - (r[54 * KQ_S] * v[155 * KQ_S]) - (r[68 * KQ_S] * v[145 * KQ_S] * v[155 * KQ_S]) - (r[70 * KQ_S] * v[157 * KQ_S]) - (r[73 * KQ_S] * v[13 * KQ_S]) - (r[76 * KQ_S] * v[12 * KQ_S]) - (r[79 * KQ_S] * v[12 * KQ_S] * v[13 * KQ_S]) - (r[81 * KQ_S] * v[120 * KQ_S] * v[155 * KQ_S]) - (r[82 * KQ_S] * v[121 * KQ_S] * v[155 * KQ_S]) - (r[83 * KQ_S] * v[121 * KQ_S]) - (r[88 * KQ_S] * v[158 * KQ_S]) - (r[90 * KQ_S] * v[149 * KQ_S]) - (r[124 * KQ_S]) - (r[236 * KQ_S] * v[160 * KQ_S]) - (r[241 * KQ_S] * v[126 * KQ_S]) - (r[245 * KQ_S] * v[127 * KQ_S] * v[155 * KQ_S]) - (r[248 * KQ_S] * v[119 * KQ_S]) - (r[250 * KQ_S] * v[143 * KQ_S]);
    jvs[658 * KQ_S] = 0.0 - (r[70 * KQ_S] * v[156 * KQ_S]);
    jvs[659 * KQ_S] = 0.0 - (r[88 * KQ_S] * v[156 * KQ_S]);
    jvs[660 * KQ_S] = 0.0 + (r[55 * KQ_S] * v[155 * KQ_S]);
    jvs[661 * KQ_S] = 0.0 - (r[236 * KQ_S] * v[156 * KQ_S]) + (r[254 * KQ_S] * v[147 * KQ_S]);
    jvs[662 * KQ_S] = 0.0 + (r[5 * KQ_S]);
    jvs[663 * KQ_S] = 0.0 - (r[69 * KQ_S] * v[157 * KQ_S]);
    jvs[664 * KQ_S] = 0.0 - (r[86 * KQ_S] * v[157 * KQ_S]);
    jvs[665 * KQ_S] = 0.0 - (r[92 * KQ_S] * v[157 * KQ_S]);
    jvs[666 * KQ_S] = 0.0;
    jvs[667 * KQ_S] = 0.0;
    jvs[668 * KQ_S] = 0.0 - (r[70 * KQ_S] * v[157 * KQ_S]);
    jvs[669 * KQ_S] = 0.0 - (r[21 * KQ_S]) - (r[69 * KQ_S] * v[144 * KQ_S]) - (r[70 * KQ_S] * v[156 * KQ_S]) - (r[71 * KQ_S] * v[159 * KQ_S]) - (r[86 * KQ_S] * v[150 * KQ_S]) - (r[92 * KQ_S] * v[151 * KQ_S]) - (r[100 * KQ_S]);
    jvs[670 * KQ_S] = 0.0;
    jvs[671 * KQ_S] = 0.0 - (r[71 * KQ_S] * v[157 * KQ_S]);
    jvs[672 * KQ_S] = 0.0;
    jvs[673 * KQ_S] = 0.0 + (r[13 * KQ_S]);
    jvs[674 * KQ_S] = 0.0 + (r[94 * KQ_S] * v[160 * KQ_S]);
    jvs[675 * KQ_S] = 0.0 + -0x1.0000000000000p+1 * (r[87 * KQ_S] * v[158 * KQ_S]);
    jvs[676 * KQ_S] = 0.0 + (r[231 * KQ_S]);
    jvs[677 * KQ_S] = 0.0 + (r[239 * KQ_S]);
    jvs[678 * KQ_S] = 0.0 - (r[238 * KQ_S] * v[158 * KQ_S]);
    jvs[679 * KQ_S] = 0.0 + (r[93 * KQ_S] * v[160 * KQ_S]);
    jvs[680 * KQ_S] = 0.0;
    jvs[681 * KQ_S] = 0.0 - (r[237 * KQ_S] * v[158 * KQ_S]);
    jvs[682 * KQ_S] = 0.0;
    jvs[683 * KQ_S] = 0.0 + -0x1.0000000000000p+1 * (r[88 * KQ_S] * v[158 * KQ_S]);
    jvs[684 * KQ_S] = 0.0;
    jvs[685 * KQ_S] = 0.0 - (r[29 * KQ_S]) + -0x1.0000000000000p+1 * (r[87 * KQ_S] * v[144 * KQ_S]) + -0x1.0000000000000p+1 * (r[88 * KQ_S] * v[156 * KQ_S]) + -0x1.0000000000000p+1 * (r[89 * KQ_S] * v[159 * KQ_S]) - (r[132 * KQ_S]) - (r[237 * KQ_S] * v[154 * KQ_S]) - (r[238 * KQ_S] * v[150 * KQ_S]);
    jvs[686 * KQ_S] = 0.0 + -0x1.0000000000000p+1 * (r[89 * KQ_S] * v[158 * KQ_S]);
    jvs[687 * KQ_S] = 0.0 + (r[93 * KQ_S] * v[151 * KQ_S]) + (r[94 * KQ_S] * v[125 * KQ_S]);
    jvs[688 * KQ_S] = 0.0 - (r[77 * KQ_S] * v[159 * KQ_S]) - (r[80 * KQ_S] * v[13 * KQ_S] * v[159 * KQ_S]);
    jvs[689 * KQ_S] = 0.0 - (r[74 * KQ_S] * v[159 * KQ_S]) - (r[80 * KQ_S] * v[12 * KQ_S] * v[159 * KQ_S]);
    jvs[690 * KQ_S] = 0.0 - (r[251 * KQ_S] * v[159 * KQ_S]);
    jvs[691 * KQ_S] = 0.0 + (r[253 * KQ_S] * v[152 * KQ_S]);
    jvs[692 * KQ_S] = 0.0;
    jvs[693 * KQ_S] = 0.0 + (r[253 * KQ_S] * v[147 * KQ_S]);
    jvs[694 * KQ_S] = 0.0;
    jvs[695 * KQ_S] = 0.0;
    jvs[696 * KQ_S] = 0.0 - (r[55 * KQ_S] * v[159 * KQ_S]);
    jvs[697 * KQ_S] = 0.0 + (r[41 * KQ_S]);
    jvs[698 * KQ_S] = 0.0 - (r[71 * KQ_S] * v[159 * KQ_S]);
    jvs[699 * KQ_S] = 0.0 - (r[89 * KQ_S] * v[159 * KQ_S]);
    jvs[700 * KQ_S] = 0.0 - (r[55 * KQ_S] * v[155 * KQ_S]) - (r[71 * KQ_S] * v[157 * KQ_S]) - (r[74 * KQ_S] * v[13 * KQ_S]) - (r[77 * KQ_S] * v[12 * KQ_S]) - (r[80 * KQ_S] * v[12 * KQ_S] * v[13 * KQ_S]) - (r[89 * KQ_S] * v[158 * KQ_S]) - (r[125 * KQ_S]) - (r[251 * KQ_S] * v[143 * KQ_S]);
    jvs[701 * KQ_S] = 0.0;
    jvs[702 * KQ_S] = 0.0 - (r[193 * KQ_S] * v[160 * KQ_S]) - (r[194 * KQ_S] * v[160 * KQ_S]);
    jvs[703 * KQ_S] = 0.0 - (r[197 * KQ_S] * v[160 * KQ_S]);
    jvs[704 * KQ_S] = 0.0 - (r[203 * KQ_S] * v[160 * KQ_S]);
}

KQ_HD KQ_NOINLINE void kqu_jac_12(const double* v, const double* f, const double* r, double* jvs)
{
    jvs[705 * KQ_S] = 0.0 + (r[246 * KQ_S] * f[0 * KQ_S]);
    jvs[706 * KQ_S] = 0.0 - (r[94 * KQ_S] * v[160 * KQ_S]);
    jvs[707 * KQ_S] = 0.0;
    jvs[708 * KQ_S] = 0.0 + -0x1.0000000000000p+1 * (r[200 * KQ_S] * v[160 * KQ_S]);
    jvs[709 * KQ_S] = 0.0 - (r[202 * KQ_S] * v[160 * KQ_S]);
    jvs[710 * KQ_S] = 0.0 - (r[201 * KQ_S] * v[160 * KQ_S]);
    jvs[711 * KQ_S] = 0.0 - (r[205 * KQ_S] * v[160 * KQ_S]);
    jvs[712 * KQ_S] = 0.0 - (r[204 * KQ_S] * v[160 * KQ_S]);
    jvs[713 * KQ_S] = 0.0 - (r[206 * KQ_S] * v[160 * KQ_S]);
    jvs[714 * KQ_S] = 0.0 - (r[207 * KQ_S] * v[160 * KQ_S]);
    jvs[715 * KQ_S] = 0.0 - (r[198 * KQ_S] * v[160 * KQ_S]);
    jvs[716 * KQ_S] = 0.0 - (r[249 * KQ_S] * v[160 * KQ_S]);
    jvs[717 * KQ_S] = 0.0 - (r[195 * KQ_S] * v[160 * KQ_S]);
    jvs[718 * KQ_S] = 0.0 - (r[196 * KQ_S] * v[160 * KQ_S]);
    jvs[719 * KQ_S] = 0.0 - (r[199 * KQ_S] * v[160 * KQ_S]);
    jvs[720 * KQ_S] = 0.0 - (r[209 * KQ_S] * v[160 * KQ_S]);
    jvs[721 * KQ_S] = 0.0;
    jvs[722 * KQ_S] = 0.0 + 0x1.0000000000000p+1 * (r[192 * KQ_S]) - (r[235 * KQ_S] * v[160 * KQ_S]);
    jvs[723 * KQ_S] = 0.0 + (r[231 * KQ_S]);
    jvs[724 * KQ_S] = 0.0 - (r[254 * KQ_S] * v[160 * KQ_S]);
    jvs[725 * KQ_S] = 0.0 - (r[208 * KQ_S] * v[160 * KQ_S]);
    jvs[726 * KQ_S] = 0.0;
    jvs[727 * KQ_S] = 0.0 + (r[86 * KQ_S] * v[157 * KQ_S]) - (r[234 * KQ_S] * v[160 * KQ_S]);
    jvs[728 * KQ_S] = 0.0 - (r[93 * KQ_S] * v[160 * KQ_S]);
    jvs[729 * KQ_S] = 0.0;
    jvs[730 * KQ_S] = 0.0;
    jvs[731 * KQ_S] = 0.0 - (r[233 * KQ_S] * v[160 * KQ_S]);
    jvs[732 * KQ_S] = 0.0;
    jvs[733 * KQ_S] = 0.0 - (r[236 * KQ_S] * v[160 * KQ_S]);
    jvs[734 * KQ_S] = 0.0 + (r[86 * KQ_S] * v[150 * KQ_S]);
    jvs[735 * KQ_S] = 0.0;
    jvs[736 * KQ_S] = 0.0;
    jvs[737 * KQ_S] = 0.0 - (r[93 * KQ_S] * v[151 * KQ_S]) - (r[94 * KQ_S] * v[125 * KQ_S]) - (r[138 * KQ_S]) - (r[139 * KQ_S]) - (r[193 * KQ_S] * v[104 * KQ_S]) - (r[194 * KQ_S] * v[104 * KQ_S]) - (r[195 * KQ_S] * v[138 * KQ_S]) - (r[196 * KQ_S] * v[139 * KQ_S]) - (r[197 * KQ_S] * v[105 * KQ_S]) - (r[198 * KQ_S] * v[136 * KQ_S]) - (r[199 * KQ_S] * v[140 * KQ_S]) + -0x1.0000000000000p+1 * (r[200 * KQ_S] * v[128 * KQ_S]) - (r[201 * KQ_S] * v[131 * KQ_S]) - (r[202 * KQ_S] * v[130 * KQ_S]) - (r[203 * KQ_S] * v[112 * KQ_S]) - (r[204 * KQ_S] * v[133 * KQ_S]) - (r[205 * KQ_S] * v[132 * KQ_S]) - (r[206 * KQ_S] * v[134 * KQ_S]) - (r[207 * KQ_S] * v[135 * KQ_S]) - (r[208 * KQ_S] * v[148 * KQ_S]) - (r[209 * KQ_S] * v[141 * KQ_S]) + -0x1.0000000000000p+1 * (r[232 * KQ_S] * 0x1.0000000000000p+1 * v[160 * KQ_S]) - (r[233 * KQ_S] * v[154 * KQ_S]) - (r[234 * KQ_S] * v[150 * KQ_S]) - (r[235 * KQ_S] * v[145 * KQ_S]) - (r[236 * KQ_S] * v[156 * KQ_S]) - (r[249 * KQ_S] * v[137 * KQ_S]) - (r[254 * KQ_S] * v[147 * KQ_S]);
}

KQ_HD inline void kqu_jac(const double* v, const double* f, const double* r, double* jvs)
{
    kqu_jac_0(v, f, r, jvs);
    kqu_jac_1(v, f, r, jvs);
    kqu_jac_2(v, f, r, jvs);
    kqu_jac_3(v, f, r, jvs);
    kqu_jac_4(v, f, r, jvs);
    kqu_jac_5(v, f, r, jvs);
    kqu_jac_6(v, f, r, jvs);
    kqu_jac_7(v, f, r, jvs);
    kqu_jac_8(v, f, r, jvs);
    kqu_jac_9(v, f, r, jvs);
    kqu_jac_10(v, f, r, jvs);
    kqu_jac_11(v, f, r, jvs);
    kqu_jac_12(v, f, r, jvs);
}

KQ_HD KQ_NOINLINE int kqu_decomp_0(double* jvs)
{
    if (fabs(jvs[0 * KQ_S]) < DBL_MIN) return 1;
    if (fabs(jvs[1 * KQ_S]) < DBL_MIN) return 2;
    if (fabs(jvs[2 * KQ_S]) < DBL_MIN) return 3;
    if (fabs(jvs[3 * KQ_S]) < DBL_MIN) return 4;
    if (fabs(jvs[4 * KQ_S]) < DBL_MIN) return 5;
    if (fabs(jvs[5 * KQ_S]) < DBL_MIN) return 6;
    if (fabs(jvs[6 * KQ_S]) < DBL_MIN) return 7;
    if (fabs(jvs[7 * KQ_S]) < DBL_MIN) return 8;
    if (fabs(jvs[9 * KQ_S]) < DBL_MIN) return 9;
    { const double a = -jvs[8 * KQ_S] / jvs[7 * KQ_S]; jvs[8 * KQ_S] = -a;
    }
    if (fabs(jvs[11 * KQ_S]) < DBL_MIN) return 10;
    { const double a = -jvs[10 * KQ_S] / jvs[5 * KQ_S]; jvs[10 * KQ_S] = -a;
    }
    if (fabs(jvs[12 * KQ_S]) < DBL_MIN) return 11;
    if (fabs(jvs[14 * KQ_S]) < DBL_MIN) return 12;
    { const double a = -jvs[13 * KQ_S] / jvs[6 * KQ_S]; jvs[13 * KQ_S] = -a;
    }
    if (fabs(jvs[15 * KQ_S]) < DBL_MIN) return 13;
    if (fabs(jvs[16 * KQ_S]) < DBL_MIN) return 14;
    if (fabs(jvs[17 * KQ_S]) < DBL_MIN) return 15;
    if (fabs(jvs[18 * KQ_S]) < DBL_MIN) return 16;
    if (fabs(jvs[19 * KQ_S]) < DBL_MIN) return 17;
    if (fabs(jvs[21 * KQ_S]) < DBL_MIN) return 18;
    { const double a = -jvs[20 * KQ_S] / jvs[3 * KQ_S]; jvs[20 * KQ_S] = -a;
    }
    if (fabs(jvs[22 * KQ_S]) < DBL_MIN) return 19;
    if (fabs(jvs[31 * KQ_S]) < DBL_MIN) return 20;
    if (fabs(jvs[33 * KQ_S]) < DBL_MIN) return 21;
    if (fabs(jvs[38 * KQ_S]) < DBL_MIN) return 22;
    if (fabs(jvs[42 * KQ_S]) < DBL_MIN) return 23;
    if (fabs(jvs[44 * KQ_S]) < DBL_MIN) return 24;
    if (fabs(jvs[46 * KQ_S]) < DBL_MIN) return 25;
    if (fabs(jvs[48 * KQ_S]) < DBL_MIN) return 26;
    if (fabs(jvs[51 * KQ_S]) < DBL_MIN) return 27;
    if (fabs(jvs[53 * KQ_S]) < DBL_MIN) return 28;
    if (fabs(jvs[55 * KQ_S]) < DBL_MIN) return 29;
    if (fabs(jvs[59 * KQ_S]) < DBL_MIN) return 30;
    if (fabs(jvs[61 * KQ_S]) < DBL_MIN) return 31;
    if (fabs(jvs[63 * KQ_S]) < DBL_MIN) return 32;
    if (fabs(jvs[65 * KQ_S]) < DBL_MIN) return 33;
    if (fabs(jvs[67 * KQ_S]) < DBL_MIN) return 34;
    if (fabs(jvs[69 * KQ_S]) < DBL_MIN) return 35;
    if (fabs(jvs[71 * KQ_S]) < DBL_MIN) return 36;
    if (fabs(jvs[74 * KQ_S]) < DBL_MIN) return 37;
    { const double a = -jvs[73 * KQ_S] / jvs[9 * KQ_S]; jvs[73 * KQ_S] = -a;
    }
    if (fabs(jvs[76 * KQ_S]) < DBL_MIN) return 38;
    { const double a = -jvs[75 * KQ_S] / jvs[15 * KQ_S]; jvs[75 * KQ_S] = -a;
    }
    if (fabs(jvs[78 * KQ_S]) < DBL_MIN) return 39;
    { const double a = -jvs[77 * KQ_S] / jvs[16 * KQ_S]; jvs[77 * KQ_S] = -a;
    }
    if (fabs(jvs[80 * KQ_S]) < DBL_MIN) return 40;
    { const double a = -jvs[79 * KQ_S] / jvs[11 * KQ_S]; jvs[79 * KQ_S] = -a;
    }
    if (fabs(jvs[82 * KQ_S]) < DBL_MIN) return 41;
    { const double a = -jvs[81 * KQ_S] / jvs[12 * KQ_S]; jvs[81 * KQ_S] = -a;
    }
    if (fabs(jvs[84 * KQ_S]) < DBL_MIN) return 42;
    { const double a = -jvs[83 * KQ_S] / jvs[14 * KQ_S]; jvs[83 * KQ_S] = -a;
    }
    if (fabs(jvs[85 * KQ_S]) < DBL_MIN) return 43;
    if (fabs(jvs[88 * KQ_S]) < DBL_MIN) return 44;
    { const double a = -jvs[87 * KQ_S] / jvs[17 * KQ_S]; jvs[87 * KQ_S] = -a;
    }
    if (fabs(jvs[90 * KQ_S]) < DBL_MIN) return 45;
    { const double a = -jvs[89 * KQ_S] / jvs[18 * KQ_S]; jvs[89 * KQ_S] = -a;
    }
    if (fabs(jvs[92 * KQ_S]) < DBL_MIN) return 46;
    { const double a = -jvs[91 * KQ_S] / jvs[19 * KQ_S]; jvs[91 * KQ_S] = -a;
    }
    if (fabs(jvs[94 * KQ_S]) < DBL_MIN) return 47;
    { const double a = -jvs[93 * KQ_S] / jvs[21 * KQ_S]; jvs[93 * KQ_S] = -a;
    }
    if (fabs(jvs[95 * KQ_S]) < DBL_MIN) return 48;
    if (fabs(jvs[97 * KQ_S]) < DBL_MIN) return 49;
    if (fabs(jvs[100 * KQ_S]) < DBL_MIN) return 50;
    if (fabs(jvs[103 * KQ_S]) < DBL_MIN) return 51;
    if (fabs(jvs[105 * KQ_S]) < DBL_MIN) return 52;
    if (fabs(jvs[108 * KQ_S]) < DBL_MIN) return 53;
    if (fabs(jvs[112 * KQ_S]) < DBL_MIN) return 54;
    if (fabs(jvs[114 * KQ_S]) < DBL_MIN) return 55;
    if (fabs(jvs[116 * KQ_S]) < DBL_MIN) return 56;
    if (fabs(jvs[120 * KQ_S]) < DBL_MIN) return 57;
    if (fabs(jvs[122 * KQ_S]) < DBL_MIN) return 58;
    if (fabs(jvs[124 * KQ_S]) < DBL_MIN) return 59;
    if (fabs(jvs[126 * KQ_S]) < DBL_MIN) return 60;
    if (fabs(jvs[129 * KQ_S]) < DBL_MIN) return 61;
    if (fabs(jvs[131 * KQ_S]) < DBL_MIN) return 62;
    if (fabs(jvs[135 * KQ_S]) < DBL_MIN) return 63;
    if (fabs(jvs[138 * KQ_S]) < DBL_MIN) return 64;
    if (fabs(jvs[142 * KQ_S]) < DBL_MIN) return 65;
    if (fabs(jvs[145 * KQ_S]) < DBL_MIN) return 66;
    if (fabs(jvs[148 * KQ_S]) < DBL_MIN) return 67;
    if (fabs(jvs[152 * KQ_S]) < DBL_MIN) return 68;
    if (fabs(jvs[155 * KQ_S]) < DBL_MIN) return 69;
    if (fabs(jvs[157 * KQ_S]) < DBL_MIN) return 70;
    if (fabs(jvs[160 * KQ_S]) < DBL_MIN) return 71;
    if (fabs(jvs[164 * KQ_S]) < DBL_MIN) return 72;
    if (fabs(jvs[166 * KQ_S]) < DBL_MIN) return 73;
    if (fabs(jvs[168 * KQ_S]) < DBL_MIN) return 74;
    if (fabs(jvs[170 * KQ_S]) < DBL_MIN) return 75;
    if (fabs(jvs[173 * KQ_S]) < DBL_MIN) return 76;
    { const double a = -jvs[172 * KQ_S] / jvs[170 * KQ_S]; jvs[172 * KQ_S] = -a;
      jvs[173 * KQ_S] = jvs[173 * KQ_S] + a * jvs[171 * KQ_S];
    }
    if (fabs(jvs[175 * KQ_S]) < DBL_MIN) return 77;
    if (fabs(jvs[178 * KQ_S]) < DBL_MIN) return 78;
    { const double a = -jvs[177 * KQ_S] / jvs[175 * KQ_S]; jvs[177 * KQ_S] = -a;
      jvs[178 * KQ_S] = jvs[178 * KQ_S] + a * jvs[176 * KQ_S];
    }
    if (fabs(jvs[180 * KQ_S]) < DBL_MIN) return 79;
    if (fabs(jvs[182 * KQ_S]) < DBL_MIN) return 80;
    if (fabs(jvs[184 * KQ_S]) < DBL_MIN) return 81;
    if (fabs(jvs[186 * KQ_S]) < DBL_MIN) return 82;
    if (fabs(jvs[188 * KQ_S]) < DBL_MIN) return 83;
    if (fabs(jvs[190 * KQ_S]) < DBL_MIN) return 84;
    if (fabs(jvs[192 * KQ_S]) < DBL_MIN) return 85;
    if (fabs(jvs[194 * KQ_S]) < DBL_MIN) return 86;
    if (fabs(jvs[196 * KQ_S]) < DBL_MIN) return 87;
    if (fabs(jvs[198 * KQ_S]) < DBL_MIN) return 88;
    if (fabs(jvs[200 * KQ_S]) < DBL_MIN) return 89;
    if (fabs(jvs[202 * KQ_S]) < DBL_MIN) return 90;
    if (fabs(jvs[204 * KQ_S]) < DBL_MIN) return 91;
    if (fabs(jvs[206 * KQ_S]) < DBL_MIN) return 92;
    if (fabs(jvs[208 * KQ_S]) < DBL_MIN) return 93;
    if (fabs(jvs[210 * KQ_S]) < DBL_MIN) return 94;
    if (fabs(jvs[212 * KQ_S]) < DBL_MIN) return 95;
    if (fabs(jvs[214 * KQ_S]) < DBL_MIN) return 96;
    if (fabs(jvs[216 * KQ_S]) < DBL_MIN) return 97;
    if (fabs(jvs[218 * KQ_S]) < DBL_MIN) return 98;
    if (fabs(jvs[220 * KQ_S]) < DBL_MIN) return 99;
    if (fabs(jvs[222 * KQ_S]) < DBL_MIN) return 100;
    if (fabs(jvs[224 * KQ_S]) < DBL_MIN) return 101;
    if (fabs(jvs[226 * KQ_S]) < DBL_MIN) return 102;
    if (fabs(jvs[228 * KQ_S]) < DBL_MIN) return 103;
    if (fabs(jvs[231 * KQ_S]) < DBL_MIN) return 104;
    if (fabs(jvs[237 * KQ_S]) < DBL_MIN) return 105;
    { const double a = -jvs[236 * KQ_S] / jvs[180 * KQ_S]; jvs[236 * KQ_S] = -a;
      jvs[237 * KQ_S] = jvs[237 * KQ_S] + a * jvs[181 * KQ_S];
    }
    if (fabs(jvs[241 * KQ_S]) < DBL_MIN) return 106;
    { const double a = -jvs[239 * KQ_S] / jvs[210 * KQ_S]; jvs[239 * KQ_S] = -a;
      jvs[241 * KQ_S] = jvs[241 * KQ_S] + a * jvs[211 * KQ_S];
    }
    { const double a = -jvs[240 * KQ_S] / jvs[237 * KQ_S]; jvs[240 * KQ_S] = -a;
      jvs[242 * KQ_S] = jvs[242 * KQ_S] + a * jvs[238 * KQ_S];
    }
    if (fabs(jvs[244 * KQ_S]) < DBL_MIN) return 107;
    { const double a = -jvs[243 * KQ_S] / jvs[194 * KQ_S]; jvs[243 * KQ_S] = -a;
      jvs[244 * KQ_S] = jvs[244 * KQ_S] + a * jvs[195 * KQ_S];
    }
    if (fabs(jvs[248 * KQ_S]) < DBL_MIN) return 108;
    { const double a = -jvs[247 * KQ_S] / jvs[198 * KQ_S]; jvs[247 * KQ_S] = -a;
      jvs[248 * KQ_S] = jvs[248 * KQ_S] + a * jvs[199 * KQ_S];
    }
    if (fabs(jvs[253 * KQ_S]) < DBL_MIN) return 109;
    { const double a = -jvs[251 * KQ_S] / jvs[1 * KQ_S]; jvs[251 * KQ_S] = -a;
    }
    { const double a = -jvs[252 * KQ_S] / jvs[248 * KQ_S]; jvs[252 * KQ_S] = -a;
      jvs[253 * KQ_S] = jvs[253 * KQ_S] + a * jvs[249 * KQ_S];
      jvs[254 * KQ_S] = jvs[254 * KQ_S] + a * jvs[250 * KQ_S];
    }
    if (fabs(jvs[255 * KQ_S]) < DBL_MIN) return 110;
    if (fabs(jvs[259 * KQ_S]) < DBL_MIN) return 111;
    { const double a = -jvs[258 * KQ_S] / jvs[208 * KQ_S]; jvs[258 * KQ_S] = -a;
      jvs[259 * KQ_S] = jvs[259 * KQ_S] + a * jvs[209 * KQ_S];
    }
    if (fabs(jvs[264 * KQ_S]) < DBL_MIN) return 112;
    { const double a = -jvs[262 * KQ_S] / jvs[2 * KQ_S]; jvs[262 * KQ_S] = -a;
    }
    { const double a = -jvs[263 * KQ_S] / jvs[259 * KQ_S]; jvs[263 * KQ_S] = -a;
      jvs[264 * KQ_S] = jvs[264 * KQ_S] + a * jvs[260 * KQ_S];
      jvs[265 * KQ_S] = jvs[265 * KQ_S] + a * jvs[261 * KQ_S];
    }
    if (fabs(jvs[267 * KQ_S]) < DBL_MIN) return 113;
    { const double a = -jvs[266 * KQ_S] / jvs[212 * KQ_S]; jvs[266 * KQ_S] = -a;
      jvs[267 * KQ_S] = jvs[267 * KQ_S] + a * jvs[213 * KQ_S];
    }
    if (fabs(jvs[269 * KQ_S]) < DBL_MIN) return 114;
    if (fabs(jvs[273 * KQ_S]) < DBL_MIN) return 115;
    { const double a = -jvs[272 * KQ_S] / jvs[269 * KQ_S]; jvs[272 * KQ_S] = -a;
      jvs[273 * KQ_S] = jvs[273 * KQ_S] + a * jvs[270 * KQ_S];
      jvs[275 * KQ_S] = jvs[275 * KQ_S] + a * jvs[271 * KQ_S];
    }
    if (fabs(jvs[279 * KQ_S]) < DBL_MIN) return 116;
    { const double a = -jvs[276 * KQ_S] / jvs[224 * KQ_S]; jvs[276 * KQ_S] = -a;
      jvs[279 * KQ_S] = jvs[279 * KQ_S] + a * jvs[225 * KQ_S];
    }
    { const double a = -jvs[277 * KQ_S] / jvs[226 * KQ_S]; jvs[277 * KQ_S] = -a;
      jvs[279 * KQ_S] = jvs[279 * KQ_S] + a * jvs[227 * KQ_S];
    }
    { const double a = -jvs[278 * KQ_S] / jvs[228 * KQ_S]; jvs[278 * KQ_S] = -a;
      jvs[279 * KQ_S] = jvs[279 * KQ_S] + a * jvs[229 * KQ_S];
      jvs[281 * KQ_S] = jvs[281 * KQ_S] + a * jvs[230 * KQ_S];
    }
    if (fabs(jvs[282 * KQ_S]) < DBL_MIN) return 117;
    if (fabs(jvs[287 * KQ_S]) < DBL_MIN) return 118;
    if (fabs(jvs[296 * KQ_S]) < DBL_MIN) return 119;
    { const double a = -jvs[293 * KQ_S] / jvs[190 * KQ_S]; jvs[293 * KQ_S] = -a;
      jvs[296 * KQ_S] = jvs[296 * KQ_S] + a * jvs[191 * KQ_S];
    }
    { const double a = -jvs[294 * KQ_S] / jvs[282 * KQ_S]; jvs[294 * KQ_S] = -a;
      jvs[295 * KQ_S] = jvs[295 * KQ_S] + a * jvs[283 * KQ_S];
      jvs[296 * KQ_S] = jvs[296 * KQ_S] + a * jvs[284 * KQ_S];
      jvs[297 * KQ_S] = jvs[297 * KQ_S] + a * jvs[285 * KQ_S];
      jvs[300 * KQ_S] = jvs[300 * KQ_S] + a * jvs[286 * KQ_S];
    }
    { const double a = -jvs[295 * KQ_S] / jvs[287 * KQ_S]; jvs[295 * KQ_S] = -a;
      jvs[296 * KQ_S] = jvs[296 * KQ_S] + a * jvs[288 * KQ_S];
      jvs[297 * KQ_S] = jvs[297 * KQ_S] + a * jvs[289 * KQ_S];
      jvs[298 * KQ_S] = jvs[298 * KQ_S] + a * jvs[290 * KQ_S];
      jvs[299 * KQ_S] = jvs[299 * KQ_S] + a * jvs[291 * KQ_S];
      jvs[300 * KQ_S] = jvs[300 * KQ_S] + a * jvs[292 * KQ_S];
    }
    if (fabs(jvs[302 * KQ_S]) < DBL_MIN) return 120;
    { const double a = -jvs[301 * KQ_S] / jvs[220 * KQ_S]; jvs[301 * KQ_S] = -a;
      jvs[302 * KQ_S] = jvs[302 * KQ_S] + a * jvs[221 * KQ_S];
    }
    if (fabs(jvs[306 * KQ_S]) < DBL_MIN) return 121;
    { const double a = -jvs[304 * KQ_S] / jvs[204 * KQ_S]; jvs[304 * KQ_S] = -a;
      jvs[306 * KQ_S] = jvs[306 * KQ_S] + a * jvs[205 * KQ_S];
    }
    { const double a = -jvs[305 * KQ_S] / jvs[302 * KQ_S]; jvs[305 * KQ_S] = -a;
      jvs[308 * KQ_S] = jvs[308 * KQ_S] + a * jvs[303 * KQ_S];
    }
    if (fabs(jvs[310 * KQ_S]) < DBL_MIN) return 122;
    { const double a = -jvs[309 * KQ_S] / jvs[206 * KQ_S]; jvs[309 * KQ_S] = -a;
      jvs[310 * KQ_S] = jvs[310 * KQ_S] + a * jvs[207 * KQ_S];
    }
    if (fabs(jvs[313 * KQ_S]) < DBL_MIN) return 123;
    return 0;
}

KQ_HD KQ_NOINLINE int kqu_decomp_1(double* jvs)
{
    if (fabs(jvs[319 * KQ_S]) < DBL_MIN) return 124;
    { const double a = -jvs[317 * KQ_S] / jvs[255 * KQ_S]; jvs[317 * KQ_S] = -a;
      jvs[319 * KQ_S] = jvs[319 * KQ_S] + a * jvs[256 * KQ_S];
      jvs[323 * KQ_S] = jvs[323 * KQ_S] + a * jvs[257 * KQ_S];
    }
    { const double a = -jvs[318 * KQ_S] / jvs[313 * KQ_S]; jvs[318 * KQ_S] = -a;
      jvs[320 * KQ_S] = jvs[320 * KQ_S] + a * jvs[314 * KQ_S];
      jvs[321 * KQ_S] = jvs[321 * KQ_S] + a * jvs[315 * KQ_S];
      jvs[322 * KQ_S] = jvs[322 * KQ_S] + a * jvs[316 * KQ_S];
    }
    if (fabs(jvs[326 * KQ_S]) < DBL_MIN) return 125;
    { const double a = -jvs[324 * KQ_S] / jvs[196 * KQ_S]; jvs[324 * KQ_S] = -a;
      jvs[326 * KQ_S] = jvs[326 * KQ_S] + a * jvs[197 * KQ_S];
    }
    { const double a = -jvs[325 * KQ_S] / jvs[273 * KQ_S]; jvs[325 * KQ_S] = -a;
      jvs[326 * KQ_S] = jvs[326 * KQ_S] + a * jvs[274 * KQ_S];
      jvs[334 * KQ_S] = jvs[334 * KQ_S] + a * jvs[275 * KQ_S];
    }
    if (fabs(jvs[337 * KQ_S]) < DBL_MIN) return 126;
    { const double a = -jvs[336 * KQ_S] / jvs[168 * KQ_S]; jvs[336 * KQ_S] = -a;
      jvs[337 * KQ_S] = jvs[337 * KQ_S] + a * jvs[169 * KQ_S];
    }
    if (fabs(jvs[342 * KQ_S]) < DBL_MIN) return 127;
    { const double a = -jvs[341 * KQ_S] / jvs[218 * KQ_S]; jvs[341 * KQ_S] = -a;
      jvs[342 * KQ_S] = jvs[342 * KQ_S] + a * jvs[219 * KQ_S];
    }
    if (fabs(jvs[345 * KQ_S]) < DBL_MIN) return 128;
    if (fabs(jvs[350 * KQ_S]) < DBL_MIN) return 129;
    if (fabs(jvs[355 * KQ_S]) < DBL_MIN) return 130;
    if (fabs(jvs[360 * KQ_S]) < DBL_MIN) return 131;
    if (fabs(jvs[366 * KQ_S]) < DBL_MIN) return 132;
    { const double a = -jvs[364 * KQ_S] / jvs[350 * KQ_S]; jvs[364 * KQ_S] = -a;
      jvs[366 * KQ_S] = jvs[366 * KQ_S] + a * jvs[351 * KQ_S];
      jvs[367 * KQ_S] = jvs[367 * KQ_S] + a * jvs[352 * KQ_S];
      jvs[369 * KQ_S] = jvs[369 * KQ_S] + a * jvs[353 * KQ_S];
      jvs[370 * KQ_S] = jvs[370 * KQ_S] + a * jvs[354 * KQ_S];
    }
    { const double a = -jvs[365 * KQ_S] / jvs[360 * KQ_S]; jvs[365 * KQ_S] = -a;
      jvs[366 * KQ_S] = jvs[366 * KQ_S] + a * jvs[361 * KQ_S];
      jvs[369 * KQ_S] = jvs[369 * KQ_S] + a * jvs[362 * KQ_S];
      jvs[370 * KQ_S] = jvs[370 * KQ_S] + a * jvs[363 * KQ_S];
    }
    if (fabs(jvs[372 * KQ_S]) < DBL_MIN) return 133;
    { const double a = -jvs[371 * KQ_S] / jvs[267 * KQ_S]; jvs[371 * KQ_S] = -a;
      jvs[375 * KQ_S] = jvs[375 * KQ_S] + a * jvs[268 * KQ_S];
    }
    if (fabs(jvs[378 * KQ_S]) < DBL_MIN) return 134;
    { const double a = -jvs[376 * KQ_S] / jvs[188 * KQ_S]; jvs[376 * KQ_S] = -a;
      jvs[378 * KQ_S] = jvs[378 * KQ_S] + a * jvs[189 * KQ_S];
    }
    { const double a = -jvs[377 * KQ_S] / jvs[372 * KQ_S]; jvs[377 * KQ_S] = -a;
      jvs[378 * KQ_S] = jvs[378 * KQ_S] + a * jvs[373 * KQ_S];
      jvs[379 * KQ_S] = jvs[379 * KQ_S] + a * jvs[374 * KQ_S];
      jvs[380 * KQ_S] = jvs[380 * KQ_S] + a * jvs[375 * KQ_S];
    }
    if (fabs(jvs[383 * KQ_S]) < DBL_MIN) return 135;
    { const double a = -jvs[381 * KQ_S] / jvs[182 * KQ_S]; jvs[381 * KQ_S] = -a;
      jvs[383 * KQ_S] = jvs[383 * KQ_S] + a * jvs[183 * KQ_S];
    }
    { const double a = -jvs[382 * KQ_S] / jvs[378 * KQ_S]; jvs[382 * KQ_S] = -a;
      jvs[385 * KQ_S] = jvs[385 * KQ_S] + a * jvs[379 * KQ_S];
      jvs[386 * KQ_S] = jvs[386 * KQ_S] + a * jvs[380 * KQ_S];
    }
    if (fabs(jvs[390 * KQ_S]) < DBL_MIN) return 136;
    { const double a = -jvs[387 * KQ_S] / jvs[372 * KQ_S]; jvs[387 * KQ_S] = -a;
      jvs[388 * KQ_S] = jvs[388 * KQ_S] + a * jvs[373 * KQ_S];
      jvs[391 * KQ_S] = jvs[391 * KQ_S] + a * jvs[374 * KQ_S];
      jvs[392 * KQ_S] = jvs[392 * KQ_S] + a * jvs[375 * KQ_S];
    }
    { const double a = -jvs[388 * KQ_S] / jvs[378 * KQ_S]; jvs[388 * KQ_S] = -a;
      jvs[391 * KQ_S] = jvs[391 * KQ_S] + a * jvs[379 * KQ_S];
      jvs[392 * KQ_S] = jvs[392 * KQ_S] + a * jvs[380 * KQ_S];
    }
    { const double a = -jvs[389 * KQ_S] / jvs[383 * KQ_S]; jvs[389 * KQ_S] = -a;
      jvs[390 * KQ_S] = jvs[390 * KQ_S] + a * jvs[384 * KQ_S];
      jvs[391 * KQ_S] = jvs[391 * KQ_S] + a * jvs[385 * KQ_S];
      jvs[392 * KQ_S] = jvs[392 * KQ_S] + a * jvs[386 * KQ_S];
    }
    if (fabs(jvs[396 * KQ_S]) < DBL_MIN) return 137;
    { const double a = -jvs[393 * KQ_S] / jvs[241 * KQ_S]; jvs[393 * KQ_S] = -a;
      jvs[399 * KQ_S] = jvs[399 * KQ_S] + a * jvs[242 * KQ_S];
    }
    { const double a = -jvs[394 * KQ_S] / jvs[383 * KQ_S]; jvs[394 * KQ_S] = -a;
      jvs[395 * KQ_S] = jvs[395 * KQ_S] + a * jvs[384 * KQ_S];
      jvs[398 * KQ_S] = jvs[398 * KQ_S] + a * jvs[385 * KQ_S];
      jvs[399 * KQ_S] = jvs[399 * KQ_S] + a * jvs[386 * KQ_S];
    }
    { const double a = -jvs[395 * KQ_S] / jvs[390 * KQ_S]; jvs[395 * KQ_S] = -a;
      jvs[398 * KQ_S] = jvs[398 * KQ_S] + a * jvs[391 * KQ_S];
      jvs[399 * KQ_S] = jvs[399 * KQ_S] + a * jvs[392 * KQ_S];
    }
    if (fabs(jvs[400 * KQ_S]) < DBL_MIN) return 138;
    if (fabs(jvs[405 * KQ_S]) < DBL_MIN) return 139;
    { const double a = -jvs[404 * KQ_S] / jvs[237 * KQ_S]; jvs[404 * KQ_S] = -a;
      jvs[408 * KQ_S] = jvs[408 * KQ_S] + a * jvs[238 * KQ_S];
    }
    if (fabs(jvs[410 * KQ_S]) < DBL_MIN) return 140;
    { const double a = -jvs[409 * KQ_S] / jvs[405 * KQ_S]; jvs[409 * KQ_S] = -a;
      jvs[410 * KQ_S] = jvs[410 * KQ_S] + a * jvs[406 * KQ_S];
      jvs[411 * KQ_S] = jvs[411 * KQ_S] + a * jvs[407 * KQ_S];
      jvs[412 * KQ_S] = jvs[412 * KQ_S] + a * jvs[408 * KQ_S];
    }
    if (fabs(jvs[418 * KQ_S]) < DBL_MIN) return 141;
    { const double a = -jvs[413 * KQ_S] / jvs[267 * KQ_S]; jvs[413 * KQ_S] = -a;
      jvs[420 * KQ_S] = jvs[420 * KQ_S] + a * jvs[268 * KQ_S];
    }
    { const double a = -jvs[414 * KQ_S] / jvs[390 * KQ_S]; jvs[414 * KQ_S] = -a;
      jvs[419 * KQ_S] = jvs[419 * KQ_S] + a * jvs[391 * KQ_S];
      jvs[420 * KQ_S] = jvs[420 * KQ_S] + a * jvs[392 * KQ_S];
    }
    { const double a = -jvs[415 * KQ_S] / jvs[396 * KQ_S]; jvs[415 * KQ_S] = -a;
      jvs[418 * KQ_S] = jvs[418 * KQ_S] + a * jvs[397 * KQ_S];
      jvs[419 * KQ_S] = jvs[419 * KQ_S] + a * jvs[398 * KQ_S];
      jvs[420 * KQ_S] = jvs[420 * KQ_S] + a * jvs[399 * KQ_S];
    }
    { const double a = -jvs[416 * KQ_S] / jvs[405 * KQ_S]; jvs[416 * KQ_S] = -a;
      jvs[417 * KQ_S] = jvs[417 * KQ_S] + a * jvs[406 * KQ_S];
      jvs[419 * KQ_S] = jvs[419 * KQ_S] + a * jvs[407 * KQ_S];
      jvs[420 * KQ_S] = jvs[420 * KQ_S] + a * jvs[408 * KQ_S];
    }
    { const double a = -jvs[417 * KQ_S] / jvs[410 * KQ_S]; jvs[417 * KQ_S] = -a;
      jvs[419 * KQ_S] = jvs[419 * KQ_S] + a * jvs[411 * KQ_S];
      jvs[420 * KQ_S] = jvs[420 * KQ_S] + a * jvs[412 * KQ_S];
    }
    if (fabs(jvs[423 * KQ_S]) < DBL_MIN) return 142;
    { const double a = -jvs[421 * KQ_S] / jvs[202 * KQ_S]; jvs[421 * KQ_S] = -a;
      jvs[423 * KQ_S] = jvs[423 * KQ_S] + a * jvs[203 * KQ_S];
    }
    { const double a = -jvs[422 * KQ_S] / jvs[400 * KQ_S]; jvs[422 * KQ_S] = -a;
      jvs[423 * KQ_S] = jvs[423 * KQ_S] + a * jvs[401 * KQ_S];
      jvs[426 * KQ_S] = jvs[426 * KQ_S] + a * jvs[402 * KQ_S];
      jvs[427 * KQ_S] = jvs[427 * KQ_S] + a * jvs[403 * KQ_S];
    }
    if (fabs(jvs[431 * KQ_S]) < DBL_MIN) return 143;
    { const double a = -jvs[428 * KQ_S] / jvs[231 * KQ_S]; jvs[428 * KQ_S] = -a;
      jvs[429 * KQ_S] = jvs[429 * KQ_S] + a * jvs[232 * KQ_S];
      jvs[430 * KQ_S] = jvs[430 * KQ_S] + a * jvs[233 * KQ_S];
      jvs[434 * KQ_S] = jvs[434 * KQ_S] + a * jvs[234 * KQ_S];
      jvs[435 * KQ_S] = jvs[435 * KQ_S] + a * jvs[235 * KQ_S];
    }
    { const double a = -jvs[429 * KQ_S] / jvs[302 * KQ_S]; jvs[429 * KQ_S] = -a;
      jvs[434 * KQ_S] = jvs[434 * KQ_S] + a * jvs[303 * KQ_S];
    }
    { const double a = -jvs[430 * KQ_S] / jvs[342 * KQ_S]; jvs[430 * KQ_S] = -a;
      jvs[432 * KQ_S] = jvs[432 * KQ_S] + a * jvs[343 * KQ_S];
      jvs[434 * KQ_S] = jvs[434 * KQ_S] + a * jvs[344 * KQ_S];
    }
    if (fabs(jvs[438 * KQ_S]) < DBL_MIN) return 144;
    { const double a = -jvs[436 * KQ_S] / jvs[184 * KQ_S]; jvs[436 * KQ_S] = -a;
      jvs[438 * KQ_S] = jvs[438 * KQ_S] + a * jvs[185 * KQ_S];
    }
    { const double a = -jvs[437 * KQ_S] / jvs[302 * KQ_S]; jvs[437 * KQ_S] = -a;
      jvs[441 * KQ_S] = jvs[441 * KQ_S] + a * jvs[303 * KQ_S];
    }
    if (fabs(jvs[446 * KQ_S]) < DBL_MIN) return 145;
    { const double a = -jvs[443 * KQ_S] / jvs[15 * KQ_S]; jvs[443 * KQ_S] = -a;
    }
    { const double a = -jvs[444 * KQ_S] / jvs[16 * KQ_S]; jvs[444 * KQ_S] = -a;
    }
    { const double a = -jvs[445 * KQ_S] / jvs[222 * KQ_S]; jvs[445 * KQ_S] = -a;
      jvs[446 * KQ_S] = jvs[446 * KQ_S] + a * jvs[223 * KQ_S];
    }
    if (fabs(jvs[452 * KQ_S]) < DBL_MIN) return 146;
    { const double a = -jvs[451 * KQ_S] / jvs[192 * KQ_S]; jvs[451 * KQ_S] = -a;
      jvs[452 * KQ_S] = jvs[452 * KQ_S] + a * jvs[193 * KQ_S];
    }
    if (fabs(jvs[462 * KQ_S]) < DBL_MIN) return 147;
    { const double a = -jvs[458 * KQ_S] / jvs[0 * KQ_S]; jvs[458 * KQ_S] = -a;
    }
    { const double a = -jvs[459 * KQ_S] / jvs[244 * KQ_S]; jvs[459 * KQ_S] = -a;
      jvs[462 * KQ_S] = jvs[462 * KQ_S] + a * jvs[245 * KQ_S];
      jvs[466 * KQ_S] = jvs[466 * KQ_S] + a * jvs[246 * KQ_S];
    }
    { const double a = -jvs[460 * KQ_S] / jvs[279 * KQ_S]; jvs[460 * KQ_S] = -a;
      jvs[462 * KQ_S] = jvs[462 * KQ_S] + a * jvs[280 * KQ_S];
      jvs[465 * KQ_S] = jvs[465 * KQ_S] + a * jvs[281 * KQ_S];
    }
    { const double a = -jvs[461 * KQ_S] / jvs[342 * KQ_S]; jvs[461 * KQ_S] = -a;
      jvs[465 * KQ_S] = jvs[465 * KQ_S] + a * jvs[343 * KQ_S];
      jvs[467 * KQ_S] = jvs[467 * KQ_S] + a * jvs[344 * KQ_S];
    }
    if (fabs(jvs[470 * KQ_S]) < DBL_MIN) return 148;
    { const double a = -jvs[469 * KQ_S] / jvs[438 * KQ_S]; jvs[469 * KQ_S] = -a;
      jvs[470 * KQ_S] = jvs[470 * KQ_S] + a * jvs[439 * KQ_S];
      jvs[471 * KQ_S] = jvs[471 * KQ_S] + a * jvs[440 * KQ_S];
      jvs[473 * KQ_S] = jvs[473 * KQ_S] + a * jvs[441 * KQ_S];
      jvs[474 * KQ_S] = jvs[474 * KQ_S] + a * jvs[442 * KQ_S];
    }
    if (fabs(jvs[480 * KQ_S]) < DBL_MIN) return 149;
    { const double a = -jvs[476 * KQ_S] / jvs[383 * KQ_S]; jvs[476 * KQ_S] = -a;
      jvs[477 * KQ_S] = jvs[477 * KQ_S] + a * jvs[384 * KQ_S];
      jvs[482 * KQ_S] = jvs[482 * KQ_S] + a * jvs[385 * KQ_S];
      jvs[485 * KQ_S] = jvs[485 * KQ_S] + a * jvs[386 * KQ_S];
    }
    { const double a = -jvs[477 * KQ_S] / jvs[390 * KQ_S]; jvs[477 * KQ_S] = -a;
      jvs[482 * KQ_S] = jvs[482 * KQ_S] + a * jvs[391 * KQ_S];
      jvs[485 * KQ_S] = jvs[485 * KQ_S] + a * jvs[392 * KQ_S];
    }
    { const double a = -jvs[478 * KQ_S] / jvs[438 * KQ_S]; jvs[478 * KQ_S] = -a;
      jvs[479 * KQ_S] = jvs[479 * KQ_S] + a * jvs[439 * KQ_S];
      jvs[480 * KQ_S] = jvs[480 * KQ_S] + a * jvs[440 * KQ_S];
      jvs[483 * KQ_S] = jvs[483 * KQ_S] + a * jvs[441 * KQ_S];
      jvs[484 * KQ_S] = jvs[484 * KQ_S] + a * jvs[442 * KQ_S];
    }
    { const double a = -jvs[479 * KQ_S] / jvs[470 * KQ_S]; jvs[479 * KQ_S] = -a;
      jvs[480 * KQ_S] = jvs[480 * KQ_S] + a * jvs[471 * KQ_S];
      jvs[481 * KQ_S] = jvs[481 * KQ_S] + a * jvs[472 * KQ_S];
      jvs[483 * KQ_S] = jvs[483 * KQ_S] + a * jvs[473 * KQ_S];
      jvs[484 * KQ_S] = jvs[484 * KQ_S] + a * jvs[474 * KQ_S];
      jvs[485 * KQ_S] = jvs[485 * KQ_S] + a * jvs[475 * KQ_S];
    }
    if (fabs(jvs[488 * KQ_S]) < DBL_MIN) return 150;
    { const double a = -jvs[486 * KQ_S] / jvs[216 * KQ_S]; jvs[486 * KQ_S] = -a;
      jvs[488 * KQ_S] = jvs[488 * KQ_S] + a * jvs[217 * KQ_S];
    }
    { const double a = -jvs[487 * KQ_S] / jvs[355 * KQ_S]; jvs[487 * KQ_S] = -a;
      jvs[488 * KQ_S] = jvs[488 * KQ_S] + a * jvs[356 * KQ_S];
      jvs[489 * KQ_S] = jvs[489 * KQ_S] + a * jvs[357 * KQ_S];
      jvs[491 * KQ_S] = jvs[491 * KQ_S] + a * jvs[358 * KQ_S];
      jvs[493 * KQ_S] = jvs[493 * KQ_S] + a * jvs[359 * KQ_S];
    }
    if (fabs(jvs[494 * KQ_S]) < DBL_MIN) return 151;
    return 0;
}

KQ_HD KQ_NOINLINE int kqu_decomp_2(double* jvs)
{
    if (fabs(jvs[505 * KQ_S]) < DBL_MIN) return 152;
    { const double a = -jvs[500 * KQ_S] / jvs[337 * KQ_S]; jvs[500 * KQ_S] = -a;
      jvs[505 * KQ_S] = jvs[505 * KQ_S] + a * jvs[338 * KQ_S];
      jvs[507 * KQ_S] = jvs[507 * KQ_S] + a * jvs[339 * KQ_S];
      jvs[512 * KQ_S] = jvs[512 * KQ_S] + a * jvs[340 * KQ_S];
    }
    { const double a = -jvs[501 * KQ_S] / jvs[355 * KQ_S]; jvs[501 * KQ_S] = -a;
      jvs[503 * KQ_S] = jvs[503 * KQ_S] + a * jvs[356 * KQ_S];
      jvs[504 * KQ_S] = jvs[504 * KQ_S] + a * jvs[357 * KQ_S];
      jvs[507 * KQ_S] = jvs[507 * KQ_S] + a * jvs[358 * KQ_S];
      jvs[510 * KQ_S] = jvs[510 * KQ_S] + a * jvs[359 * KQ_S];
    }
    { const double a = -jvs[502 * KQ_S] / jvs[446 * KQ_S]; jvs[502 * KQ_S] = -a;
      jvs[507 * KQ_S] = jvs[507 * KQ_S] + a * jvs[447 * KQ_S];
      jvs[508 * KQ_S] = jvs[508 * KQ_S] + a * jvs[448 * KQ_S];
      jvs[509 * KQ_S] = jvs[509 * KQ_S] + a * jvs[449 * KQ_S];
      jvs[510 * KQ_S] = jvs[510 * KQ_S] + a * jvs[450 * KQ_S];
    }
    { const double a = -jvs[503 * KQ_S] / jvs[488 * KQ_S]; jvs[503 * KQ_S] = -a;
      jvs[504 * KQ_S] = jvs[504 * KQ_S] + a * jvs[489 * KQ_S];
      jvs[506 * KQ_S] = jvs[506 * KQ_S] + a * jvs[490 * KQ_S];
      jvs[507 * KQ_S] = jvs[507 * KQ_S] + a * jvs[491 * KQ_S];
      jvs[508 * KQ_S] = jvs[508 * KQ_S] + a * jvs[492 * KQ_S];
      jvs[510 * KQ_S] = jvs[510 * KQ_S] + a * jvs[493 * KQ_S];
    }
    { const double a = -jvs[504 * KQ_S] / jvs[494 * KQ_S]; jvs[504 * KQ_S] = -a;
      jvs[506 * KQ_S] = jvs[506 * KQ_S] + a * jvs[495 * KQ_S];
      jvs[507 * KQ_S] = jvs[507 * KQ_S] + a * jvs[496 * KQ_S];
      jvs[509 * KQ_S] = jvs[509 * KQ_S] + a * jvs[497 * KQ_S];
      jvs[510 * KQ_S] = jvs[510 * KQ_S] + a * jvs[498 * KQ_S];
      jvs[512 * KQ_S] = jvs[512 * KQ_S] + a * jvs[499 * KQ_S];
    }
    if (fabs(jvs[528 * KQ_S]) < DBL_MIN) return 153;
    { const double a = -jvs[513 * KQ_S] / jvs[248 * KQ_S]; jvs[513 * KQ_S] = -a;
      jvs[514 * KQ_S] = jvs[514 * KQ_S] + a * jvs[249 * KQ_S];
      jvs[528 * KQ_S] = jvs[528 * KQ_S] + a * jvs[250 * KQ_S];
    }
    { const double a = -jvs[514 * KQ_S] / jvs[253 * KQ_S]; jvs[514 * KQ_S] = -a;
      jvs[528 * KQ_S] = jvs[528 * KQ_S] + a * jvs[254 * KQ_S];
    }
    { const double a = -jvs[515 * KQ_S] / jvs[360 * KQ_S]; jvs[515 * KQ_S] = -a;
      jvs[516 * KQ_S] = jvs[516 * KQ_S] + a * jvs[361 * KQ_S];
      jvs[531 * KQ_S] = jvs[531 * KQ_S] + a * jvs[362 * KQ_S];
      jvs[536 * KQ_S] = jvs[536 * KQ_S] + a * jvs[363 * KQ_S];
    }
    { const double a = -jvs[516 * KQ_S] / jvs[366 * KQ_S]; jvs[516 * KQ_S] = -a;
      jvs[517 * KQ_S] = jvs[517 * KQ_S] + a * jvs[367 * KQ_S];
      jvs[519 * KQ_S] = jvs[519 * KQ_S] + a * jvs[368 * KQ_S];
      jvs[531 * KQ_S] = jvs[531 * KQ_S] + a * jvs[369 * KQ_S];
      jvs[536 * KQ_S] = jvs[536 * KQ_S] + a * jvs[370 * KQ_S];
    }
    { const double a = -jvs[517 * KQ_S] / jvs[396 * KQ_S]; jvs[517 * KQ_S] = -a;
      jvs[519 * KQ_S] = jvs[519 * KQ_S] + a * jvs[397 * KQ_S];
      jvs[531 * KQ_S] = jvs[531 * KQ_S] + a * jvs[398 * KQ_S];
      jvs[536 * KQ_S] = jvs[536 * KQ_S] + a * jvs[399 * KQ_S];
    }
    { const double a = -jvs[518 * KQ_S] / jvs[400 * KQ_S]; jvs[518 * KQ_S] = -a;
      jvs[520 * KQ_S] = jvs[520 * KQ_S] + a * jvs[401 * KQ_S];
      jvs[531 * KQ_S] = jvs[531 * KQ_S] + a * jvs[402 * KQ_S];
      jvs[536 * KQ_S] = jvs[536 * KQ_S] + a * jvs[403 * KQ_S];
    }
    { const double a = -jvs[519 * KQ_S] / jvs[418 * KQ_S]; jvs[519 * KQ_S] = -a;
      jvs[531 * KQ_S] = jvs[531 * KQ_S] + a * jvs[419 * KQ_S];
      jvs[536 * KQ_S] = jvs[536 * KQ_S] + a * jvs[420 * KQ_S];
    }
    { const double a = -jvs[520 * KQ_S] / jvs[423 * KQ_S]; jvs[520 * KQ_S] = -a;
      jvs[523 * KQ_S] = jvs[523 * KQ_S] + a * jvs[424 * KQ_S];
      jvs[524 * KQ_S] = jvs[524 * KQ_S] + a * jvs[425 * KQ_S];
      jvs[531 * KQ_S] = jvs[531 * KQ_S] + a * jvs[426 * KQ_S];
      jvs[536 * KQ_S] = jvs[536 * KQ_S] + a * jvs[427 * KQ_S];
    }
    { const double a = -jvs[521 * KQ_S] / jvs[438 * KQ_S]; jvs[521 * KQ_S] = -a;
      jvs[523 * KQ_S] = jvs[523 * KQ_S] + a * jvs[439 * KQ_S];
      jvs[524 * KQ_S] = jvs[524 * KQ_S] + a * jvs[440 * KQ_S];
      jvs[532 * KQ_S] = jvs[532 * KQ_S] + a * jvs[441 * KQ_S];
      jvs[535 * KQ_S] = jvs[535 * KQ_S] + a * jvs[442 * KQ_S];
    }
    { const double a = -jvs[522 * KQ_S] / jvs[462 * KQ_S]; jvs[522 * KQ_S] = -a;
      jvs[525 * KQ_S] = jvs[525 * KQ_S] + a * jvs[463 * KQ_S];
      jvs[527 * KQ_S] = jvs[527 * KQ_S] + a * jvs[464 * KQ_S];
      jvs[529 * KQ_S] = jvs[529 * KQ_S] + a * jvs[465 * KQ_S];
      jvs[531 * KQ_S] = jvs[531 * KQ_S] + a * jvs[466 * KQ_S];
      jvs[532 * KQ_S] = jvs[532 * KQ_S] + a * jvs[467 * KQ_S];
      jvs[533 * KQ_S] = jvs[533 * KQ_S] + a * jvs[468 * KQ_S];
    }
    { const double a = -jvs[523 * KQ_S] / jvs[470 * KQ_S]; jvs[523 * KQ_S] = -a;
      jvs[524 * KQ_S] = jvs[524 * KQ_S] + a * jvs[471 * KQ_S];
      jvs[528 * KQ_S] = jvs[528 * KQ_S] + a * jvs[472 * KQ_S];
      jvs[532 * KQ_S] = jvs[532 * KQ_S] + a * jvs[473 * KQ_S];
      jvs[535 * KQ_S] = jvs[535 * KQ_S] + a * jvs[474 * KQ_S];
      jvs[536 * KQ_S] = jvs[536 * KQ_S] + a * jvs[475 * KQ_S];
    }
    { const double a = -jvs[524 * KQ_S] / jvs[480 * KQ_S]; jvs[524 * KQ_S] = -a;
      jvs[528 * KQ_S] = jvs[528 * KQ_S] + a * jvs[481 * KQ_S];
      jvs[531 * KQ_S] = jvs[531 * KQ_S] + a * jvs[482 * KQ_S];
      jvs[532 * KQ_S] = jvs[532 * KQ_S] + a * jvs[483 * KQ_S];
      jvs[535 * KQ_S] = jvs[535 * KQ_S] + a * jvs[484 * KQ_S];
      jvs[536 * KQ_S] = jvs[536 * KQ_S] + a * jvs[485 * KQ_S];
    }
    { const double a = -jvs[525 * KQ_S] / jvs[488 * KQ_S]; jvs[525 * KQ_S] = -a;
      jvs[526 * KQ_S] = jvs[526 * KQ_S] + a * jvs[489 * KQ_S];
      jvs[530 * KQ_S] = jvs[530 * KQ_S] + a * jvs[490 * KQ_S];
      jvs[531 * KQ_S] = jvs[531 * KQ_S] + a * jvs[491 * KQ_S];
      jvs[532 * KQ_S] = jvs[532 * KQ_S] + a * jvs[492 * KQ_S];
      jvs[534 * KQ_S] = jvs[534 * KQ_S] + a * jvs[493 * KQ_S];
    }
    { const double a = -jvs[526 * KQ_S] / jvs[494 * KQ_S]; jvs[526 * KQ_S] = -a;
      jvs[530 * KQ_S] = jvs[530 * KQ_S] + a * jvs[495 * KQ_S];
      jvs[531 * KQ_S] = jvs[531 * KQ_S] + a * jvs[496 * KQ_S];
      jvs[533 * KQ_S] = jvs[533 * KQ_S] + a * jvs[497 * KQ_S];
      jvs[534 * KQ_S] = jvs[534 * KQ_S] + a * jvs[498 * KQ_S];
      jvs[536 * KQ_S] = jvs[536 * KQ_S] + a * jvs[499 * KQ_S];
    }
    { const double a = -jvs[527 * KQ_S] / jvs[505 * KQ_S]; jvs[527 * KQ_S] = -a;
      jvs[530 * KQ_S] = jvs[530 * KQ_S] + a * jvs[506 * KQ_S];
      jvs[531 * KQ_S] = jvs[531 * KQ_S] + a * jvs[507 * KQ_S];
      jvs[532 * KQ_S] = jvs[532 * KQ_S] + a * jvs[508 * KQ_S];
      jvs[533 * KQ_S] = jvs[533 * KQ_S] + a * jvs[509 * KQ_S];
      jvs[534 * KQ_S] = jvs[534 * KQ_S] + a * jvs[510 * KQ_S];
      jvs[535 * KQ_S] = jvs[535 * KQ_S] + a * jvs[511 * KQ_S];
      jvs[536 * KQ_S] = jvs[536 * KQ_S] + a * jvs[512 * KQ_S];
    }
    if (fabs(jvs[555 * KQ_S]) < DBL_MIN) return 154;
    { const double a = -jvs[537 * KQ_S] / jvs[4 * KQ_S]; jvs[537 * KQ_S] = -a;
    }
    { const double a = -jvs[538 * KQ_S] / jvs[15 * KQ_S]; jvs[538 * KQ_S] = -a;
    }
    { const double a = -jvs[539 * KQ_S] / jvs[16 * KQ_S]; jvs[539 * KQ_S] = -a;
    }
    { const double a = -jvs[540 * KQ_S] / jvs[173 * KQ_S]; jvs[540 * KQ_S] = -a;
      jvs[555 * KQ_S] = jvs[555 * KQ_S] + a * jvs[174 * KQ_S];
    }
    { const double a = -jvs[541 * KQ_S] / jvs[178 * KQ_S]; jvs[541 * KQ_S] = -a;
      jvs[555 * KQ_S] = jvs[555 * KQ_S] + a * jvs[179 * KQ_S];
    }
    { const double a = -jvs[542 * KQ_S] / jvs[279 * KQ_S]; jvs[542 * KQ_S] = -a;
      jvs[551 * KQ_S] = jvs[551 * KQ_S] + a * jvs[280 * KQ_S];
      jvs[555 * KQ_S] = jvs[555 * KQ_S] + a * jvs[281 * KQ_S];
    }
    { const double a = -jvs[543 * KQ_S] / jvs[306 * KQ_S]; jvs[543 * KQ_S] = -a;
      jvs[557 * KQ_S] = jvs[557 * KQ_S] + a * jvs[307 * KQ_S];
      jvs[558 * KQ_S] = jvs[558 * KQ_S] + a * jvs[308 * KQ_S];
    }
    { const double a = -jvs[544 * KQ_S] / jvs[310 * KQ_S]; jvs[544 * KQ_S] = -a;
      jvs[557 * KQ_S] = jvs[557 * KQ_S] + a * jvs[311 * KQ_S];
      jvs[558 * KQ_S] = jvs[558 * KQ_S] + a * jvs[312 * KQ_S];
    }
    { const double a = -jvs[545 * KQ_S] / jvs[319 * KQ_S]; jvs[545 * KQ_S] = -a;
      jvs[546 * KQ_S] = jvs[546 * KQ_S] + a * jvs[320 * KQ_S];
      jvs[548 * KQ_S] = jvs[548 * KQ_S] + a * jvs[321 * KQ_S];
      jvs[555 * KQ_S] = jvs[555 * KQ_S] + a * jvs[322 * KQ_S];
      jvs[557 * KQ_S] = jvs[557 * KQ_S] + a * jvs[323 * KQ_S];
    }
    { const double a = -jvs[546 * KQ_S] / jvs[342 * KQ_S]; jvs[546 * KQ_S] = -a;
      jvs[555 * KQ_S] = jvs[555 * KQ_S] + a * jvs[343 * KQ_S];
      jvs[558 * KQ_S] = jvs[558 * KQ_S] + a * jvs[344 * KQ_S];
    }
    { const double a = -jvs[547 * KQ_S] / jvs[345 * KQ_S]; jvs[547 * KQ_S] = -a;
      jvs[548 * KQ_S] = jvs[548 * KQ_S] + a * jvs[346 * KQ_S];
      jvs[556 * KQ_S] = jvs[556 * KQ_S] + a * jvs[347 * KQ_S];
      jvs[557 * KQ_S] = jvs[557 * KQ_S] + a * jvs[348 * KQ_S];
      jvs[558 * KQ_S] = jvs[558 * KQ_S] + a * jvs[349 * KQ_S];
    }
    { const double a = -jvs[548 * KQ_S] / jvs[431 * KQ_S]; jvs[548 * KQ_S] = -a;
      jvs[555 * KQ_S] = jvs[555 * KQ_S] + a * jvs[432 * KQ_S];
      jvs[556 * KQ_S] = jvs[556 * KQ_S] + a * jvs[433 * KQ_S];
      jvs[558 * KQ_S] = jvs[558 * KQ_S] + a * jvs[434 * KQ_S];
      jvs[562 * KQ_S] = jvs[562 * KQ_S] + a * jvs[435 * KQ_S];
    }
    { const double a = -jvs[549 * KQ_S] / jvs[446 * KQ_S]; jvs[549 * KQ_S] = -a;
      jvs[557 * KQ_S] = jvs[557 * KQ_S] + a * jvs[447 * KQ_S];
      jvs[558 * KQ_S] = jvs[558 * KQ_S] + a * jvs[448 * KQ_S];
      jvs[559 * KQ_S] = jvs[559 * KQ_S] + a * jvs[449 * KQ_S];
      jvs[560 * KQ_S] = jvs[560 * KQ_S] + a * jvs[450 * KQ_S];
    }
    { const double a = -jvs[550 * KQ_S] / jvs[452 * KQ_S]; jvs[550 * KQ_S] = -a;
      jvs[553 * KQ_S] = jvs[553 * KQ_S] + a * jvs[453 * KQ_S];
      jvs[556 * KQ_S] = jvs[556 * KQ_S] + a * jvs[454 * KQ_S];
      jvs[557 * KQ_S] = jvs[557 * KQ_S] + a * jvs[455 * KQ_S];
      jvs[558 * KQ_S] = jvs[558 * KQ_S] + a * jvs[456 * KQ_S];
      jvs[562 * KQ_S] = jvs[562 * KQ_S] + a * jvs[457 * KQ_S];
    }
    { const double a = -jvs[551 * KQ_S] / jvs[462 * KQ_S]; jvs[551 * KQ_S] = -a;
      jvs[552 * KQ_S] = jvs[552 * KQ_S] + a * jvs[463 * KQ_S];
      jvs[554 * KQ_S] = jvs[554 * KQ_S] + a * jvs[464 * KQ_S];
      jvs[555 * KQ_S] = jvs[555 * KQ_S] + a * jvs[465 * KQ_S];
      jvs[557 * KQ_S] = jvs[557 * KQ_S] + a * jvs[466 * KQ_S];
      jvs[558 * KQ_S] = jvs[558 * KQ_S] + a * jvs[467 * KQ_S];
      jvs[559 * KQ_S] = jvs[559 * KQ_S] + a * jvs[468 * KQ_S];
    }
    { const double a = -jvs[552 * KQ_S] / jvs[488 * KQ_S]; jvs[552 * KQ_S] = -a;
      jvs[553 * KQ_S] = jvs[553 * KQ_S] + a * jvs[489 * KQ_S];
      jvs[556 * KQ_S] = jvs[556 * KQ_S] + a * jvs[490 * KQ_S];
      jvs[557 * KQ_S] = jvs[557 * KQ_S] + a * jvs[491 * KQ_S];
      jvs[558 * KQ_S] = jvs[558 * KQ_S] + a * jvs[492 * KQ_S];
      jvs[560 * KQ_S] = jvs[560 * KQ_S] + a * jvs[493 * KQ_S];
    }
    { const double a = -jvs[553 * KQ_S] / jvs[494 * KQ_S]; jvs[553 * KQ_S] = -a;
      jvs[556 * KQ_S] = jvs[556 * KQ_S] + a * jvs[495 * KQ_S];
      jvs[557 * KQ_S] = jvs[557 * KQ_S] + a * jvs[496 * KQ_S];
      jvs[559 * KQ_S] = jvs[559 * KQ_S] + a * jvs[497 * KQ_S];
      jvs[560 * KQ_S] = jvs[560 * KQ_S] + a * jvs[498 * KQ_S];
      jvs[562 * KQ_S] = jvs[562 * KQ_S] + a * jvs[499 * KQ_S];
    }
    { const double a = -jvs[554 * KQ_S] / jvs[505 * KQ_S]; jvs[554 * KQ_S] = -a;
      jvs[556 * KQ_S] = jvs[556 * KQ_S] + a * jvs[506 * KQ_S];
      jvs[557 * KQ_S] = jvs[557 * KQ_S] + a * jvs[507 * KQ_S];
      jvs[558 * KQ_S] = jvs[558 * KQ_S] + a * jvs[508 * KQ_S];
      jvs[559 * KQ_S] = jvs[559 * KQ_S] + a * jvs[509 * KQ_S];
      jvs[560 * KQ_S] = jvs[560 * KQ_S] + a * jvs[510 * KQ_S];
      jvs[561 * KQ_S] = jvs[561 * KQ_S] + a * jvs[511 * KQ_S];
      jvs[562 * KQ_S] = jvs[562 * KQ_S] + a * jvs[512 * KQ_S];
    }
    return 0;
}

KQ_HD KQ_NOINLINE int kqu_decomp_3(double* jvs)
{
    if (fabs(jvs[584 * KQ_S]) < DBL_MIN) return 155;
    { const double a = -jvs[563 * KQ_S] / jvs[186 * KQ_S]; jvs[563 * KQ_S] = -a;
      jvs[584 * KQ_S] = jvs[584 * KQ_S] + a * jvs[187 * KQ_S];
    }
    { const double a = -jvs[564 * KQ_S] / jvs[237 * KQ_S]; jvs[564 * KQ_S] = -a;
      jvs[590 * KQ_S] = jvs[590 * KQ_S] + a * jvs[238 * KQ_S];
    }
    { const double a = -jvs[565 * KQ_S] / jvs[241 * KQ_S]; jvs[565 * KQ_S] = -a;
      jvs[590 * KQ_S] = jvs[590 * KQ_S] + a * jvs[242 * KQ_S];
    }
    { const double a = -jvs[566 * KQ_S] / jvs[267 * KQ_S]; jvs[566 * KQ_S] = -a;
      jvs[590 * KQ_S] = jvs[590 * KQ_S] + a * jvs[268 * KQ_S];
    }
    { const double a = -jvs[567 * KQ_S] / jvs[302 * KQ_S]; jvs[567 * KQ_S] = -a;
      jvs[586 * KQ_S] = jvs[586 * KQ_S] + a * jvs[303 * KQ_S];
    }
    { const double a = -jvs[568 * KQ_S] / jvs[372 * KQ_S]; jvs[568 * KQ_S] = -a;
      jvs[569 * KQ_S] = jvs[569 * KQ_S] + a * jvs[373 * KQ_S];
      jvs[585 * KQ_S] = jvs[585 * KQ_S] + a * jvs[374 * KQ_S];
      jvs[590 * KQ_S] = jvs[590 * KQ_S] + a * jvs[375 * KQ_S];
    }
    { const double a = -jvs[569 * KQ_S] / jvs[378 * KQ_S]; jvs[569 * KQ_S] = -a;
      jvs[585 * KQ_S] = jvs[585 * KQ_S] + a * jvs[379 * KQ_S];
      jvs[590 * KQ_S] = jvs[590 * KQ_S] + a * jvs[380 * KQ_S];
    }
    { const double a = -jvs[570 * KQ_S] / jvs[396 * KQ_S]; jvs[570 * KQ_S] = -a;
      jvs[574 * KQ_S] = jvs[574 * KQ_S] + a * jvs[397 * KQ_S];
      jvs[585 * KQ_S] = jvs[585 * KQ_S] + a * jvs[398 * KQ_S];
      jvs[590 * KQ_S] = jvs[590 * KQ_S] + a * jvs[399 * KQ_S];
    }
    { const double a = -jvs[571 * KQ_S] / jvs[400 * KQ_S]; jvs[571 * KQ_S] = -a;
      jvs[575 * KQ_S] = jvs[575 * KQ_S] + a * jvs[401 * KQ_S];
      jvs[585 * KQ_S] = jvs[585 * KQ_S] + a * jvs[402 * KQ_S];
      jvs[590 * KQ_S] = jvs[590 * KQ_S] + a * jvs[403 * KQ_S];
    }
    { const double a = -jvs[572 * KQ_S] / jvs[405 * KQ_S]; jvs[572 * KQ_S] = -a;
      jvs[573 * KQ_S] = jvs[573 * KQ_S] + a * jvs[406 * KQ_S];
      jvs[585 * KQ_S] = jvs[585 * KQ_S] + a * jvs[407 * KQ_S];
      jvs[590 * KQ_S] = jvs[590 * KQ_S] + a * jvs[408 * KQ_S];
    }
    { const double a = -jvs[573 * KQ_S] / jvs[410 * KQ_S]; jvs[573 * KQ_S] = -a;
      jvs[585 * KQ_S] = jvs[585 * KQ_S] + a * jvs[411 * KQ_S];
      jvs[590 * KQ_S] = jvs[590 * KQ_S] + a * jvs[412 * KQ_S];
    }
    { const double a = -jvs[574 * KQ_S] / jvs[418 * KQ_S]; jvs[574 * KQ_S] = -a;
      jvs[585 * KQ_S] = jvs[585 * KQ_S] + a * jvs[419 * KQ_S];
      jvs[590 * KQ_S] = jvs[590 * KQ_S] + a * jvs[420 * KQ_S];
    }
    { const double a = -jvs[575 * KQ_S] / jvs[423 * KQ_S]; jvs[575 * KQ_S] = -a;
      jvs[578 * KQ_S] = jvs[578 * KQ_S] + a * jvs[424 * KQ_S];
      jvs[579 * KQ_S] = jvs[579 * KQ_S] + a * jvs[425 * KQ_S];
      jvs[585 * KQ_S] = jvs[585 * KQ_S] + a * jvs[426 * KQ_S];
      jvs[590 * KQ_S] = jvs[590 * KQ_S] + a * jvs[427 * KQ_S];
    }
    { const double a = -jvs[576 * KQ_S] / jvs[431 * KQ_S]; jvs[576 * KQ_S] = -a;
      jvs[583 * KQ_S] = jvs[583 * KQ_S] + a * jvs[432 * KQ_S];
      jvs[584 * KQ_S] = jvs[584 * KQ_S] + a * jvs[433 * KQ_S];
      jvs[586 * KQ_S] = jvs[586 * KQ_S] + a * jvs[434 * KQ_S];
      jvs[590 * KQ_S] = jvs[590 * KQ_S] + a * jvs[435 * KQ_S];
    }
    { const double a = -jvs[577 * KQ_S] / jvs[452 * KQ_S]; jvs[577 * KQ_S] = -a;
      jvs[581 * KQ_S] = jvs[581 * KQ_S] + a * jvs[453 * KQ_S];
      jvs[584 * KQ_S] = jvs[584 * KQ_S] + a * jvs[454 * KQ_S];
      jvs[585 * KQ_S] = jvs[585 * KQ_S] + a * jvs[455 * KQ_S];
      jvs[586 * KQ_S] = jvs[586 * KQ_S] + a * jvs[456 * KQ_S];
      jvs[590 * KQ_S] = jvs[590 * KQ_S] + a * jvs[457 * KQ_S];
    }
    { const double a = -jvs[578 * KQ_S] / jvs[470 * KQ_S]; jvs[578 * KQ_S] = -a;
      jvs[579 * KQ_S] = jvs[579 * KQ_S] + a * jvs[471 * KQ_S];
      jvs[582 * KQ_S] = jvs[582 * KQ_S] + a * jvs[472 * KQ_S];
      jvs[586 * KQ_S] = jvs[586 * KQ_S] + a * jvs[473 * KQ_S];
      jvs[589 * KQ_S] = jvs[589 * KQ_S] + a * jvs[474 * KQ_S];
      jvs[590 * KQ_S] = jvs[590 * KQ_S] + a * jvs[475 * KQ_S];
    }
    { const double a = -jvs[579 * KQ_S] / jvs[480 * KQ_S]; jvs[579 * KQ_S] = -a;
      jvs[582 * KQ_S] = jvs[582 * KQ_S] + a * jvs[481 * KQ_S];
      jvs[585 * KQ_S] = jvs[585 * KQ_S] + a * jvs[482 * KQ_S];
      jvs[586 * KQ_S] = jvs[586 * KQ_S] + a * jvs[483 * KQ_S];
      jvs[589 * KQ_S] = jvs[589 * KQ_S] + a * jvs[484 * KQ_S];
      jvs[590 * KQ_S] = jvs[590 * KQ_S] + a * jvs[485 * KQ_S];
    }
    { const double a = -jvs[580 * KQ_S] / jvs[488 * KQ_S]; jvs[580 * KQ_S] = -a;
      jvs[581 * KQ_S] = jvs[581 * KQ_S] + a * jvs[489 * KQ_S];
      jvs[584 * KQ_S] = jvs[584 * KQ_S] + a * jvs[490 * KQ_S];
      jvs[585 * KQ_S] = jvs[585 * KQ_S] + a * jvs[491 * KQ_S];
      jvs[586 * KQ_S] = jvs[586 * KQ_S] + a * jvs[492 * KQ_S];
      jvs[588 * KQ_S] = jvs[588 * KQ_S] + a * jvs[493 * KQ_S];
    }
    { const double a = -jvs[581 * KQ_S] / jvs[494 * KQ_S]; jvs[581 * KQ_S] = -a;
      jvs[584 * KQ_S] = jvs[584 * KQ_S] + a * jvs[495 * KQ_S];
      jvs[585 * KQ_S] = jvs[585 * KQ_S] + a * jvs[496 * KQ_S];
      jvs[587 * KQ_S] = jvs[587 * KQ_S] + a * jvs[497 * KQ_S];
      jvs[588 * KQ_S] = jvs[588 * KQ_S] + a * jvs[498 * KQ_S];
      jvs[590 * KQ_S] = jvs[590 * KQ_S] + a * jvs[499 * KQ_S];
    }
    { const double a = -jvs[582 * KQ_S] / jvs[528 * KQ_S]; jvs[582 * KQ_S] = -a;
      jvs[583 * KQ_S] = jvs[583 * KQ_S] + a * jvs[529 * KQ_S];
      jvs[584 * KQ_S] = jvs[584 * KQ_S] + a * jvs[530 * KQ_S];
      jvs[585 * KQ_S] = jvs[585 * KQ_S] + a * jvs[531 * KQ_S];
      jvs[586 * KQ_S] = jvs[586 * KQ_S] + a * jvs[532 * KQ_S];
      jvs[587 * KQ_S] = jvs[587 * KQ_S] + a * jvs[533 * KQ_S];
      jvs[588 * KQ_S] = jvs[588 * KQ_S] + a * jvs[534 * KQ_S];
      jvs[589 * KQ_S] = jvs[589 * KQ_S] + a * jvs[535 * KQ_S];
      jvs[590 * KQ_S] = jvs[590 * KQ_S] + a * jvs[536 * KQ_S];
    }
    { const double a = -jvs[583 * KQ_S] / jvs[555 * KQ_S]; jvs[583 * KQ_S] = -a;
      jvs[584 * KQ_S] = jvs[584 * KQ_S] + a * jvs[556 * KQ_S];
      jvs[585 * KQ_S] = jvs[585 * KQ_S] + a * jvs[557 * KQ_S];
      jvs[586 * KQ_S] = jvs[586 * KQ_S] + a * jvs[558 * KQ_S];
      jvs[587 * KQ_S] = jvs[587 * KQ_S] + a * jvs[559 * KQ_S];
      jvs[588 * KQ_S] = jvs[588 * KQ_S] + a * jvs[560 * KQ_S];
      jvs[589 * KQ_S] = jvs[589 * KQ_S] + a * jvs[561 * KQ_S];
      jvs[590 * KQ_S] = jvs[590 * KQ_S] + a * jvs[562 * KQ_S];
    }
    return 0;
}

KQ_HD KQ_NOINLINE int kqu_decomp_4(double* jvs)
{
    if (fabs(jvs[632 * KQ_S]) < DBL_MIN) return 156;
    { const double a = -jvs[591 * KQ_S] / jvs[15 * KQ_S]; jvs[591 * KQ_S] = -a;
    }
    { const double a = -jvs[592 * KQ_S] / jvs[16 * KQ_S]; jvs[592 * KQ_S] = -a;
    }
    { const double a = -jvs[593 * KQ_S] / jvs[244 * KQ_S]; jvs[593 * KQ_S] = -a;
      jvs[623 * KQ_S] = jvs[623 * KQ_S] + a * jvs[245 * KQ_S];
      jvs[632 * KQ_S] = jvs[632 * KQ_S] + a * jvs[246 * KQ_S];
    }
    { const double a = -jvs[594 * KQ_S] / jvs[255 * KQ_S]; jvs[594 * KQ_S] = -a;
      jvs[601 * KQ_S] = jvs[601 * KQ_S] + a * jvs[256 * KQ_S];
      jvs[632 * KQ_S] = jvs[632 * KQ_S] + a * jvs[257 * KQ_S];
    }
    { const double a = -jvs[595 * KQ_S] / jvs[259 * KQ_S]; jvs[595 * KQ_S] = -a;
      jvs[596 * KQ_S] = jvs[596 * KQ_S] + a * jvs[260 * KQ_S];
      jvs[632 * KQ_S] = jvs[632 * KQ_S] + a * jvs[261 * KQ_S];
    }
    { const double a = -jvs[596 * KQ_S] / jvs[264 * KQ_S]; jvs[596 * KQ_S] = -a;
      jvs[632 * KQ_S] = jvs[632 * KQ_S] + a * jvs[265 * KQ_S];
    }
    { const double a = -jvs[597 * KQ_S] / jvs[269 * KQ_S]; jvs[597 * KQ_S] = -a;
      jvs[598 * KQ_S] = jvs[598 * KQ_S] + a * jvs[270 * KQ_S];
      jvs[632 * KQ_S] = jvs[632 * KQ_S] + a * jvs[271 * KQ_S];
    }
    { const double a = -jvs[598 * KQ_S] / jvs[273 * KQ_S]; jvs[598 * KQ_S] = -a;
      jvs[602 * KQ_S] = jvs[602 * KQ_S] + a * jvs[274 * KQ_S];
      jvs[632 * KQ_S] = jvs[632 * KQ_S] + a * jvs[275 * KQ_S];
    }
    { const double a = -jvs[599 * KQ_S] / jvs[306 * KQ_S]; jvs[599 * KQ_S] = -a;
      jvs[632 * KQ_S] = jvs[632 * KQ_S] + a * jvs[307 * KQ_S];
      jvs[633 * KQ_S] = jvs[633 * KQ_S] + a * jvs[308 * KQ_S];
    }
    { const double a = -jvs[600 * KQ_S] / jvs[310 * KQ_S]; jvs[600 * KQ_S] = -a;
      jvs[632 * KQ_S] = jvs[632 * KQ_S] + a * jvs[311 * KQ_S];
      jvs[633 * KQ_S] = jvs[633 * KQ_S] + a * jvs[312 * KQ_S];
    }
    { const double a = -jvs[601 * KQ_S] / jvs[319 * KQ_S]; jvs[601 * KQ_S] = -a;
      jvs[604 * KQ_S] = jvs[604 * KQ_S] + a * jvs[320 * KQ_S];
      jvs[620 * KQ_S] = jvs[620 * KQ_S] + a * jvs[321 * KQ_S];
      jvs[630 * KQ_S] = jvs[630 * KQ_S] + a * jvs[322 * KQ_S];
      jvs[632 * KQ_S] = jvs[632 * KQ_S] + a * jvs[323 * KQ_S];
    }
    { const double a = -jvs[602 * KQ_S] / jvs[326 * KQ_S]; jvs[602 * KQ_S] = -a;
      jvs[606 * KQ_S] = jvs[606 * KQ_S] + a * jvs[327 * KQ_S];
      jvs[608 * KQ_S] = jvs[608 * KQ_S] + a * jvs[328 * KQ_S];
      jvs[609 * KQ_S] = jvs[609 * KQ_S] + a * jvs[329 * KQ_S];
      jvs[610 * KQ_S] = jvs[610 * KQ_S] + a * jvs[330 * KQ_S];
      jvs[611 * KQ_S] = jvs[611 * KQ_S] + a * jvs[331 * KQ_S];
      jvs[615 * KQ_S] = jvs[615 * KQ_S] + a * jvs[332 * KQ_S];
      jvs[619 * KQ_S] = jvs[619 * KQ_S] + a * jvs[333 * KQ_S];
      jvs[632 * KQ_S] = jvs[632 * KQ_S] + a * jvs[334 * KQ_S];
      jvs[637 * KQ_S] = jvs[637 * KQ_S] + a * jvs[335 * KQ_S];
    }
    { const double a = -jvs[603 * KQ_S] / jvs[337 * KQ_S]; jvs[603 * KQ_S] = -a;
      jvs[628 * KQ_S] = jvs[628 * KQ_S] + a * jvs[338 * KQ_S];
      jvs[632 * KQ_S] = jvs[632 * KQ_S] + a * jvs[339 * KQ_S];
      jvs[637 * KQ_S] = jvs[637 * KQ_S] + a * jvs[340 * KQ_S];
    }
    { const double a = -jvs[604 * KQ_S] / jvs[342 * KQ_S]; jvs[604 * KQ_S] = -a;
      jvs[630 * KQ_S] = jvs[630 * KQ_S] + a * jvs[343 * KQ_S];
      jvs[633 * KQ_S] = jvs[633 * KQ_S] + a * jvs[344 * KQ_S];
    }
    { const double a = -jvs[605 * KQ_S] / jvs[345 * KQ_S]; jvs[605 * KQ_S] = -a;
      jvs[620 * KQ_S] = jvs[620 * KQ_S] + a * jvs[346 * KQ_S];
      jvs[631 * KQ_S] = jvs[631 * KQ_S] + a * jvs[347 * KQ_S];
      jvs[632 * KQ_S] = jvs[632 * KQ_S] + a * jvs[348 * KQ_S];
      jvs[633 * KQ_S] = jvs[633 * KQ_S] + a * jvs[349 * KQ_S];
    }
    { const double a = -jvs[606 * KQ_S] / jvs[350 * KQ_S]; jvs[606 * KQ_S] = -a;
      jvs[609 * KQ_S] = jvs[609 * KQ_S] + a * jvs[351 * KQ_S];
      jvs[614 * KQ_S] = jvs[614 * KQ_S] + a * jvs[352 * KQ_S];
      jvs[632 * KQ_S] = jvs[632 * KQ_S] + a * jvs[353 * KQ_S];
      jvs[637 * KQ_S] = jvs[637 * KQ_S] + a * jvs[354 * KQ_S];
    }
    { const double a = -jvs[607 * KQ_S] / jvs[355 * KQ_S]; jvs[607 * KQ_S] = -a;
      jvs[626 * KQ_S] = jvs[626 * KQ_S] + a * jvs[356 * KQ_S];
      jvs[627 * KQ_S] = jvs[627 * KQ_S] + a * jvs[357 * KQ_S];
      jvs[632 * KQ_S] = jvs[632 * KQ_S] + a * jvs[358 * KQ_S];
      jvs[635 * KQ_S] = jvs[635 * KQ_S] + a * jvs[359 * KQ_S];
    }
    { const double a = -jvs[608 * KQ_S] / jvs[360 * KQ_S]; jvs[608 * KQ_S] = -a;
      jvs[609 * KQ_S] = jvs[609 * KQ_S] + a * jvs[361 * KQ_S];
      jvs[632 * KQ_S] = jvs[632 * KQ_S] + a * jvs[362 * KQ_S];
      jvs[637 * KQ_S] = jvs[637 * KQ_S] + a * jvs[363 * KQ_S];
    }
    { const double a = -jvs[609 * KQ_S] / jvs[366 * KQ_S]; jvs[609 * KQ_S] = -a;
      jvs[614 * KQ_S] = jvs[614 * KQ_S] + a * jvs[367 * KQ_S];
      jvs[618 * KQ_S] = jvs[618 * KQ_S] + a * jvs[368 * KQ_S];
      jvs[632 * KQ_S] = jvs[632 * KQ_S] + a * jvs[369 * KQ_S];
      jvs[637 * KQ_S] = jvs[637 * KQ_S] + a * jvs[370 * KQ_S];
    }
    { const double a = -jvs[610 * KQ_S] / jvs[372 * KQ_S]; jvs[610 * KQ_S] = -a;
      jvs[611 * KQ_S] = jvs[611 * KQ_S] + a * jvs[373 * KQ_S];
      jvs[632 * KQ_S] = jvs[632 * KQ_S] + a * jvs[374 * KQ_S];
      jvs[637 * KQ_S] = jvs[637 * KQ_S] + a * jvs[375 * KQ_S];
    }
    { const double a = -jvs[611 * KQ_S] / jvs[378 * KQ_S]; jvs[611 * KQ_S] = -a;
      jvs[632 * KQ_S] = jvs[632 * KQ_S] + a * jvs[379 * KQ_S];
      jvs[637 * KQ_S] = jvs[637 * KQ_S] + a * jvs[380 * KQ_S];
    }
    { const double a = -jvs[612 * KQ_S] / jvs[383 * KQ_S]; jvs[612 * KQ_S] = -a;
      jvs[613 * KQ_S] = jvs[613 * KQ_S] + a * jvs[384 * KQ_S];
      jvs[632 * KQ_S] = jvs[632 * KQ_S] + a * jvs[385 * KQ_S];
      jvs[637 * KQ_S] = jvs[637 * KQ_S] + a * jvs[386 * KQ_S];
    }
    { const double a = -jvs[613 * KQ_S] / jvs[390 * KQ_S]; jvs[613 * KQ_S] = -a;
      jvs[632 * KQ_S] = jvs[632 * KQ_S] + a * jvs[391 * KQ_S];
      jvs[637 * KQ_S] = jvs[637 * KQ_S] + a * jvs[392 * KQ_S];
    }
    { const double a = -jvs[614 * KQ_S] / jvs[396 * KQ_S]; jvs[614 * KQ_S] = -a;
      jvs[618 * KQ_S] = jvs[618 * KQ_S] + a * jvs[397 * KQ_S];
      jvs[632 * KQ_S] = jvs[632 * KQ_S] + a * jvs[398 * KQ_S];
      jvs[637 * KQ_S] = jvs[637 * KQ_S] + a * jvs[399 * KQ_S];
    }
    { const double a = -jvs[615 * KQ_S] / jvs[400 * KQ_S]; jvs[615 * KQ_S] = -a;
      jvs[619 * KQ_S] = jvs[619 * KQ_S] + a * jvs[401 * KQ_S];
      jvs[632 * KQ_S] = jvs[632 * KQ_S] + a * jvs[402 * KQ_S];
      jvs[637 * KQ_S] = jvs[637 * KQ_S] + a * jvs[403 * KQ_S];
    }
    { const double a = -jvs[616 * KQ_S] / jvs[405 * KQ_S]; jvs[616 * KQ_S] = -a;
      jvs[617 * KQ_S] = jvs[617 * KQ_S] + a * jvs[406 * KQ_S];
      jvs[632 * KQ_S] = jvs[632 * KQ_S] + a * jvs[407 * KQ_S];
      jvs[637 * KQ_S] = jvs[637 * KQ_S] + a * jvs[408 * KQ_S];
    }
    { const double a = -jvs[617 * KQ_S] / jvs[410 * KQ_S]; jvs[617 * KQ_S] = -a;
      jvs[632 * KQ_S] = jvs[632 * KQ_S] + a * jvs[411 * KQ_S];
      jvs[637 * KQ_S] = jvs[637 * KQ_S] + a * jvs[412 * KQ_S];
    }
    { const double a = -jvs[618 * KQ_S] / jvs[418 * KQ_S]; jvs[618 * KQ_S] = -a;
      jvs[632 * KQ_S] = jvs[632 * KQ_S] + a * jvs[419 * KQ_S];
      jvs[637 * KQ_S] = jvs[637 * KQ_S] + a * jvs[420 * KQ_S];
    }
    { const double a = -jvs[619 * KQ_S] / jvs[423 * KQ_S]; jvs[619 * KQ_S] = -a;
      jvs[624 * KQ_S] = jvs[624 * KQ_S] + a * jvs[424 * KQ_S];
      jvs[625 * KQ_S] = jvs[625 * KQ_S] + a * jvs[425 * KQ_S];
      jvs[632 * KQ_S] = jvs[632 * KQ_S] + a * jvs[426 * KQ_S];
      jvs[637 * KQ_S] = jvs[637 * KQ_S] + a * jvs[427 * KQ_S];
    }
    { const double a = -jvs[620 * KQ_S] / jvs[431 * KQ_S]; jvs[620 * KQ_S] = -a;
      jvs[630 * KQ_S] = jvs[630 * KQ_S] + a * jvs[432 * KQ_S];
      jvs[631 * KQ_S] = jvs[631 * KQ_S] + a * jvs[433 * KQ_S];
      jvs[633 * KQ_S] = jvs[633 * KQ_S] + a * jvs[434 * KQ_S];
      jvs[637 * KQ_S] = jvs[637 * KQ_S] + a * jvs[435 * KQ_S];
    }
    { const double a = -jvs[621 * KQ_S] / jvs[446 * KQ_S]; jvs[621 * KQ_S] = -a;
      jvs[632 * KQ_S] = jvs[632 * KQ_S] + a * jvs[447 * KQ_S];
      jvs[633 * KQ_S] = jvs[633 * KQ_S] + a * jvs[448 * KQ_S];
      jvs[634 * KQ_S] = jvs[634 * KQ_S] + a * jvs[449 * KQ_S];
      jvs[635 * KQ_S] = jvs[635 * KQ_S] + a * jvs[450 * KQ_S];
    }
    { const double a = -jvs[622 * KQ_S] / jvs[452 * KQ_S]; jvs[622 * KQ_S] = -a;
      jvs[627 * KQ_S] = jvs[627 * KQ_S] + a * jvs[453 * KQ_S];
      jvs[631 * KQ_S] = jvs[631 * KQ_S] + a * jvs[454 * KQ_S];
      jvs[632 * KQ_S] = jvs[632 * KQ_S] + a * jvs[455 * KQ_S];
      jvs[633 * KQ_S] = jvs[633 * KQ_S] + a * jvs[456 * KQ_S];
      jvs[637 * KQ_S] = jvs[637 * KQ_S] + a * jvs[457 * KQ_S];
    }
    { const double a = -jvs[623 * KQ_S] / jvs[462 * KQ_S]; jvs[623 * KQ_S] = -a;
      jvs[626 * KQ_S] = jvs[626 * KQ_S] + a * jvs[463 * KQ_S];
      jvs[628 * KQ_S] = jvs[628 * KQ_S] + a * jvs[464 * KQ_S];
      jvs[630 * KQ_S] = jvs[630 * KQ_S] + a * jvs[465 * KQ_S];
      jvs[632 * KQ_S] = jvs[632 * KQ_S] + a * jvs[466 * KQ_S];
      jvs[633 * KQ_S] = jvs[633 * KQ_S] + a * jvs[467 * KQ_S];
      jvs[634 * KQ_S] = jvs[634 * KQ_S] + a * jvs[468 * KQ_S];
    }
    { const double a = -jvs[624 * KQ_S] / jvs[470 * KQ_S]; jvs[624 * KQ_S] = -a;
      jvs[625 * KQ_S] = jvs[625 * KQ_S] + a * jvs[471 * KQ_S];
      jvs[629 * KQ_S] = jvs[629 * KQ_S] + a * jvs[472 * KQ_S];
      jvs[633 * KQ_S] = jvs[633 * KQ_S] + a * jvs[473 * KQ_S];
      jvs[636 * KQ_S] = jvs[636 * KQ_S] + a * jvs[474 * KQ_S];
      jvs[637 * KQ_S] = jvs[637 * KQ_S] + a * jvs[475 * KQ_S];
    }
    { const double a = -jvs[625 * KQ_S] / jvs[480 * KQ_S]; jvs[625 * KQ_S] = -a;
      jvs[629 * KQ_S] = jvs[629 * KQ_S] + a * jvs[481 * KQ_S];
      jvs[632 * KQ_S] = jvs[632 * KQ_S] + a * jvs[482 * KQ_S];
      jvs[633 * KQ_S] = jvs[633 * KQ_S] + a * jvs[483 * KQ_S];
      jvs[636 * KQ_S] = jvs[636 * KQ_S] + a * jvs[484 * KQ_S];
      jvs[637 * KQ_S] = jvs[637 * KQ_S] + a * jvs[485 * KQ_S];
    }
    { const double a = -jvs[626 * KQ_S] / jvs[488 * KQ_S]; jvs[626 * KQ_S] = -a;
      jvs[627 * KQ_S] = jvs[627 * KQ_S] + a * jvs[489 * KQ_S];
      jvs[631 * KQ_S] = jvs[631 * KQ_S] + a * jvs[490 * KQ_S];
      jvs[632 * KQ_S] = jvs[632 * KQ_S] + a * jvs[491 * KQ_S];
      jvs[633 * KQ_S] = jvs[633 * KQ_S] + a * jvs[492 * KQ_S];
      jvs[635 * KQ_S] = jvs[635 * KQ_S] + a * jvs[493 * KQ_S];
    }
    { const double a = -jvs[627 * KQ_S] / jvs[494 * KQ_S]; jvs[627 * KQ_S] = -a;
      jvs[631 * KQ_S] = jvs[631 * KQ_S] + a * jvs[495 * KQ_S];
      jvs[632 * KQ_S] = jvs[632 * KQ_S] + a * jvs[496 * KQ_S];
      jvs[634 * KQ_S] = jvs[634 * KQ_S] + a * jvs[497 * KQ_S];
      jvs[635 * KQ_S] = jvs[635 * KQ_S] + a * jvs[498 * KQ_S];
      jvs[637 * KQ_S] = jvs[637 * KQ_S] + a * jvs[499 * KQ_S];
    }
    { const double a = -jvs[628 * KQ_S] / jvs[505 * KQ_S]; jvs[628 * KQ_S] = -a;
      jvs[631 * KQ_S] = jvs[631 * KQ_S] + a * jvs[506 * KQ_S];
      jvs[632 * KQ_S] = jvs[632 * KQ_S] + a * jvs[507 * KQ_S];
      jvs[633 * KQ_S] = jvs[633 * KQ_S] + a * jvs[508 * KQ_S];
      jvs[634 * KQ_S] = jvs[634 * KQ_S] + a * jvs[509 * KQ_S];
      jvs[635 * KQ_S] = jvs[635 * KQ_S] + a * jvs[510 * KQ_S];
      jvs[636 * KQ_S] = jvs[636 * KQ_S] + a * jvs[511 * KQ_S];
      jvs[637 * KQ_S] = jvs[637 * KQ_S] + a * jvs[512 * KQ_S];
    }
    { const double a = -jvs[629 * KQ_S] / jvs[528 * KQ_S]; jvs[629 * KQ_S] = -a;
      jvs[630 * KQ_S] = jvs[630 * KQ_S] + a * jvs[529 * KQ_S];
      jvs[631 * KQ_S] = jvs[631 * KQ_S] + a * jvs[530 * KQ_S];
      jvs[632 * KQ_S] = jvs[632 * KQ_S] + a * jvs[531 * KQ_S];
      jvs[633 * KQ_S] = jvs[633 * KQ_S] + a * jvs[532 * KQ_S];
      jvs[634 * KQ_S] = jvs[634 * KQ_S] + a * jvs[533 * KQ_S];
      jvs[635 * KQ_S] = jvs[635 * KQ_S] + a * jvs[534 * KQ_S];
      jvs[636 * KQ_S] = jvs[636 * KQ_S] + a * jvs[535 * KQ_S];
      jvs[637 * KQ_S] = jvs[637 * KQ_S] + a * jvs[536 * KQ_S];
    }
    { const double a = -jvs[630 * KQ_S] / jvs[555 * KQ_S]; jvs[630 * KQ_S] = -a;
      jvs[631 * KQ_S] = jvs[631 * KQ_S] + a * jvs[556 * KQ_S];
      jvs[632 * KQ_S] = jvs[632 * KQ_S] + a * jvs[557 * KQ_S];
      jvs[633 * KQ_S] = jvs[633 * KQ_S] + a * jvs[558 * KQ_S];
      jvs[634 * KQ_S] = jvs[634 * KQ_S] + a * jvs[559 * KQ_S];
      jvs[635 * KQ_S] = jvs[635 * KQ_S] + a * jvs[560 * KQ_S];
      jvs[636 * KQ_S] = jvs[636 * KQ_S] + a * jvs[561 * KQ_S];
      jvs[637 * KQ_S] = jvs[637 * KQ_S] + a * jvs[562 * KQ_S];
    }
    { const double a = -jvs[631 * KQ_S] / jvs[584 * KQ_S]; jvs[631 * KQ_S] = -a;
      jvs[632 * KQ_S] = jvs[632 * KQ_S] + a * jvs[585 * KQ_S];
      jvs[633 * KQ_S] = jvs[633 * KQ_S] + a * jvs[586 * KQ_S];
      jvs[634 * KQ_S] = jvs[634 * KQ_S] + a * jvs[587 * KQ_S];
      jvs[635 * KQ_S] = jvs[635 * KQ_S] + a * jvs[588 * KQ_S];
      jvs[636 * KQ_S] = jvs[636 * KQ_S] + a * jvs[589 * KQ_S];
      jvs[637 * KQ_S] = jvs[637 * KQ_S] + a * jvs[590 * KQ_S];
    }
    return 0;
}

KQ_HD KQ_NOINLINE int kqu_decomp_5(double* jvs)
{
    if (fabs(jvs[657 * KQ_S]) < DBL_MIN) return 157;
    { const double a = -jvs[638 * KQ_S] / jvs[15 * KQ_S]; jvs[638 * KQ_S] = -a;
    }
    { const double a = -jvs[639 * KQ_S] / jvs[16 * KQ_S]; jvs[639 * KQ_S] = -a;
    }
    { const double a = -jvs[640 * KQ_S] / jvs[302 * KQ_S]; jvs[640 * KQ_S] = -a;
      jvs[657 * KQ_S] = jvs[657 * KQ_S] + a * jvs[303 * KQ_S];
    }
    { const double a = -jvs[641 * KQ_S] / jvs[306 * KQ_S]; jvs[641 * KQ_S] = -a;
      jvs[656 * KQ_S] = jvs[656 * KQ_S] + a * jvs[307 * KQ_S];
      jvs[657 * KQ_S] = jvs[657 * KQ_S] + a * jvs[308 * KQ_S];
    }
    { const double a = -jvs[642 * KQ_S] / jvs[310 * KQ_S]; jvs[642 * KQ_S] = -a;
      jvs[656 * KQ_S] = jvs[656 * KQ_S] + a * jvs[311 * KQ_S];
      jvs[657 * KQ_S] = jvs[657 * KQ_S] + a * jvs[312 * KQ_S];
    }
    { const double a = -jvs[643 * KQ_S] / jvs[342 * KQ_S]; jvs[643 * KQ_S] = -a;
      jvs[654 * KQ_S] = jvs[654 * KQ_S] + a * jvs[343 * KQ_S];
      jvs[657 * KQ_S] = jvs[657 * KQ_S] + a * jvs[344 * KQ_S];
    }
    { const double a = -jvs[644 * KQ_S] / jvs[345 * KQ_S]; jvs[644 * KQ_S] = -a;
      jvs[645 * KQ_S] = jvs[645 * KQ_S] + a * jvs[346 * KQ_S];
      jvs[655 * KQ_S] = jvs[655 * KQ_S] + a * jvs[347 * KQ_S];
      jvs[656 * KQ_S] = jvs[656 * KQ_S] + a * jvs[348 * KQ_S];
      jvs[657 * KQ_S] = jvs[657 * KQ_S] + a * jvs[349 * KQ_S];
    }
    { const double a = -jvs[645 * KQ_S] / jvs[431 * KQ_S]; jvs[645 * KQ_S] = -a;
      jvs[654 * KQ_S] = jvs[654 * KQ_S] + a * jvs[432 * KQ_S];
      jvs[655 * KQ_S] = jvs[655 * KQ_S] + a * jvs[433 * KQ_S];
      jvs[657 * KQ_S] = jvs[657 * KQ_S] + a * jvs[434 * KQ_S];
      jvs[661 * KQ_S] = jvs[661 * KQ_S] + a * jvs[435 * KQ_S];
    }
    { const double a = -jvs[646 * KQ_S] / jvs[438 * KQ_S]; jvs[646 * KQ_S] = -a;
      jvs[649 * KQ_S] = jvs[649 * KQ_S] + a * jvs[439 * KQ_S];
      jvs[650 * KQ_S] = jvs[650 * KQ_S] + a * jvs[440 * KQ_S];
      jvs[657 * KQ_S] = jvs[657 * KQ_S] + a * jvs[441 * KQ_S];
      jvs[660 * KQ_S] = jvs[660 * KQ_S] + a * jvs[442 * KQ_S];
    }
    { const double a = -jvs[647 * KQ_S] / jvs[446 * KQ_S]; jvs[647 * KQ_S] = -a;
      jvs[656 * KQ_S] = jvs[656 * KQ_S] + a * jvs[447 * KQ_S];
      jvs[657 * KQ_S] = jvs[657 * KQ_S] + a * jvs[448 * KQ_S];
      jvs[658 * KQ_S] = jvs[658 * KQ_S] + a * jvs[449 * KQ_S];
      jvs[659 * KQ_S] = jvs[659 * KQ_S] + a * jvs[450 * KQ_S];
    }
    { const double a = -jvs[648 * KQ_S] / jvs[452 * KQ_S]; jvs[648 * KQ_S] = -a;
      jvs[652 * KQ_S] = jvs[652 * KQ_S] + a * jvs[453 * KQ_S];
      jvs[655 * KQ_S] = jvs[655 * KQ_S] + a * jvs[454 * KQ_S];
      jvs[656 * KQ_S] = jvs[656 * KQ_S] + a * jvs[455 * KQ_S];
      jvs[657 * KQ_S] = jvs[657 * KQ_S] + a * jvs[456 * KQ_S];
      jvs[661 * KQ_S] = jvs[661 * KQ_S] + a * jvs[457 * KQ_S];
    }
    { const double a = -jvs[649 * KQ_S] / jvs[470 * KQ_S]; jvs[649 * KQ_S] = -a;
      jvs[650 * KQ_S] = jvs[650 * KQ_S] + a * jvs[471 * KQ_S];
      jvs[653 * KQ_S] = jvs[653 * KQ_S] + a * jvs[472 * KQ_S];
      jvs[657 * KQ_S] = jvs[657 * KQ_S] + a * jvs[473 * KQ_S];
      jvs[660 * KQ_S] = jvs[660 * KQ_S] + a * jvs[474 * KQ_S];
      jvs[661 * KQ_S] = jvs[661 * KQ_S] + a * jvs[475 * KQ_S];
    }
    { const double a = -jvs[650 * KQ_S] / jvs[480 * KQ_S]; jvs[650 * KQ_S] = -a;
      jvs[653 * KQ_S] = jvs[653 * KQ_S] + a * jvs[481 * KQ_S];
      jvs[656 * KQ_S] = jvs[656 * KQ_S] + a * jvs[482 * KQ_S];
      jvs[657 * KQ_S] = jvs[657 * KQ_S] + a * jvs[483 * KQ_S];
      jvs[660 * KQ_S] = jvs[660 * KQ_S] + a * jvs[484 * KQ_S];
      jvs[661 * KQ_S] = jvs[661 * KQ_S] + a * jvs[485 * KQ_S];
    }
    { const double a = -jvs[651 * KQ_S] / jvs[488 * KQ_S]; jvs[651 * KQ_S] = -a;
      jvs[652 * KQ_S] = jvs[652 * KQ_S] + a * jvs[489 * KQ_S];
      jvs[655 * KQ_S] = jvs[655 * KQ_S] + a * jvs[490 * KQ_S];
      jvs[656 * KQ_S] = jvs[656 * KQ_S] + a * jvs[491 * KQ_S];
      jvs[657 * KQ_S] = jvs[657 * KQ_S] + a * jvs[492 * KQ_S];
      jvs[659 * KQ_S] = jvs[659 * KQ_S] + a * jvs[493 * KQ_S];
    }
    { const double a = -jvs[652 * KQ_S] / jvs[494 * KQ_S]; jvs[652 * KQ_S] = -a;
      jvs[655 * KQ_S] = jvs[655 * KQ_S] + a * jvs[495 * KQ_S];
      jvs[656 * KQ_S] = jvs[656 * KQ_S] + a * jvs[496 * KQ_S];
      jvs[658 * KQ_S] = jvs[658 * KQ_S] + a * jvs[497 * KQ_S];
      jvs[659 * KQ_S] = jvs[659 * KQ_S] + a * jvs[498 * KQ_S];
      jvs[661 * KQ_S] = jvs[661 * KQ_S] + a * jvs[499 * KQ_S];
    }
    { const double a = -jvs[653 * KQ_S] / jvs[528 * KQ_S]; jvs[653 * KQ_S] = -a;
      jvs[654 * KQ_S] = jvs[654 * KQ_S] + a * jvs[529 * KQ_S];
      jvs[655 * KQ_S] = jvs[655 * KQ_S] + a * jvs[530 * KQ_S];
      jvs[656 * KQ_S] = jvs[656 * KQ_S] + a * jvs[531 * KQ_S];
      jvs[657 * KQ_S] = jvs[657 * KQ_S] + a * jvs[532 * KQ_S];
      jvs[658 * KQ_S] = jvs[658 * KQ_S] + a * jvs[533 * KQ_S];
      jvs[659 * KQ_S] = jvs[659 * KQ_S] + a * jvs[534 * KQ_S];
      jvs[660 * KQ_S] = jvs[660 * KQ_S] + a * jvs[535 * KQ_S];
      jvs[661 * KQ_S] = jvs[661 * KQ_S] + a * jvs[536 * KQ_S];
    }
    { const double a = -jvs[654 * KQ_S] / jvs[555 * KQ_S]; jvs[654 * KQ_S] = -a;
      jvs[655 * KQ_S] = jvs[655 * KQ_S] + a * jvs[556 * KQ_S];
      jvs[656 * KQ_S] = jvs[656 * KQ_S] + a * jvs[557 * KQ_S];
      jvs[657 * KQ_S] = jvs[657 * KQ_S] + a * jvs[558 * KQ_S];
      jvs[658 * KQ_S] = jvs[658 * KQ_S] + a * jvs[559 * KQ_S];
      jvs[659 * KQ_S] = jvs[659 * KQ_S] + a * jvs[560 * KQ_S];
      jvs[660 * KQ_S] = jvs[660 * KQ_S] + a * jvs[561 * KQ_S];
      jvs[661 * KQ_S] = jvs[661 * KQ_S] + a * jvs[562 * KQ_S];
    }
    { const double a = -jvs[655 * KQ_S] / jvs[584 * KQ_S]; jvs[655 * KQ_S] = -a;
      jvs[656 * KQ_S] = jvs[656 * KQ_S] + a * jvs[585 * KQ_S];
      jvs[657 * KQ_S] = jvs[657 * KQ_S] + a * jvs[586 * KQ_S];
      jvs[658 * KQ_S] = jvs[658 * KQ_S] + a * jvs[587 * KQ_S];
      jvs[659 * KQ_S] = jvs[659 * KQ_S] + a * jvs[588 * KQ_S];
      jvs[660 * KQ_S] = jvs[660 * KQ_S] + a * jvs[589 * KQ_S];
      jvs[661 * KQ_S] = jvs[661 * KQ_S] + a * jvs[590 * KQ_S];
    }
    { const double a = -jvs[656 * KQ_S] / jvs[632 * KQ_S]; jvs[656 * KQ_S] = -a;
      jvs[657 * KQ_S] = jvs[657 * KQ_S] + a * jvs[633 * KQ_S];
      jvs[658 * KQ_S] = jvs[658 * KQ_S] + a * jvs[634 * KQ_S];
      jvs[659 * KQ_S] = jvs[659 * KQ_S] + a * jvs[635 * KQ_S];
      jvs[660 * KQ_S] = jvs[660 * KQ_S] + a * jvs[636 * KQ_S];
      jvs[661 * KQ_S] = jvs[661 * KQ_S] + a * jvs[637 * KQ_S];
    }
    if (fabs(jvs[669 * KQ_S]) < DBL_MIN) return 158;
    { const double a = -jvs[662 * KQ_S] / jvs[200 * KQ_S]; jvs[662 * KQ_S] = -a;
      jvs[669 * KQ_S] = jvs[669 * KQ_S] + a * jvs[201 * KQ_S];
    }
    { const double a = -jvs[663 * KQ_S] / jvs[446 * KQ_S]; jvs[663 * KQ_S] = -a;
      jvs[667 * KQ_S] = jvs[667 * KQ_S] + a * jvs[447 * KQ_S];
      jvs[668 * KQ_S] = jvs[668 * KQ_S] + a * jvs[448 * KQ_S];
      jvs[669 * KQ_S] = jvs[669 * KQ_S] + a * jvs[449 * KQ_S];
      jvs[670 * KQ_S] = jvs[670 * KQ_S] + a * jvs[450 * KQ_S];
    }
    { const double a = -jvs[664 * KQ_S] / jvs[494 * KQ_S]; jvs[664 * KQ_S] = -a;
      jvs[666 * KQ_S] = jvs[666 * KQ_S] + a * jvs[495 * KQ_S];
      jvs[667 * KQ_S] = jvs[667 * KQ_S] + a * jvs[496 * KQ_S];
      jvs[669 * KQ_S] = jvs[669 * KQ_S] + a * jvs[497 * KQ_S];
      jvs[670 * KQ_S] = jvs[670 * KQ_S] + a * jvs[498 * KQ_S];
      jvs[672 * KQ_S] = jvs[672 * KQ_S] + a * jvs[499 * KQ_S];
    }
    { const double a = -jvs[665 * KQ_S] / jvs[505 * KQ_S]; jvs[665 * KQ_S] = -a;
      jvs[666 * KQ_S] = jvs[666 * KQ_S] + a * jvs[506 * KQ_S];
      jvs[667 * KQ_S] = jvs[667 * KQ_S] + a * jvs[507 * KQ_S];
      jvs[668 * KQ_S] = jvs[668 * KQ_S] + a * jvs[508 * KQ_S];
      jvs[669 * KQ_S] = jvs[669 * KQ_S] + a * jvs[509 * KQ_S];
      jvs[670 * KQ_S] = jvs[670 * KQ_S] + a * jvs[510 * KQ_S];
      jvs[671 * KQ_S] = jvs[671 * KQ_S] + a * jvs[511 * KQ_S];
      jvs[672 * KQ_S] = jvs[672 * KQ_S] + a * jvs[512 * KQ_S];
    }
    { const double a = -jvs[666 * KQ_S] / jvs[584 * KQ_S]; jvs[666 * KQ_S] = -a;
      jvs[667 * KQ_S] = jvs[667 * KQ_S] + a * jvs[585 * KQ_S];
      jvs[668 * KQ_S] = jvs[668 * KQ_S] + a * jvs[586 * KQ_S];
      jvs[669 * KQ_S] = jvs[669 * KQ_S] + a * jvs[587 * KQ_S];
      jvs[670 * KQ_S] = jvs[670 * KQ_S] + a * jvs[588 * KQ_S];
      jvs[671 * KQ_S] = jvs[671 * KQ_S] + a * jvs[589 * KQ_S];
      jvs[672 * KQ_S] = jvs[672 * KQ_S] + a * jvs[590 * KQ_S];
    }
    { const double a = -jvs[667 * KQ_S] / jvs[632 * KQ_S]; jvs[667 * KQ_S] = -a;
      jvs[668 * KQ_S] = jvs[668 * KQ_S] + a * jvs[633 * KQ_S];
      jvs[669 * KQ_S] = jvs[669 * KQ_S] + a * jvs[634 * KQ_S];
      jvs[670 * KQ_S] = jvs[670 * KQ_S] + a * jvs[635 * KQ_S];
      jvs[671 * KQ_S] = jvs[671 * KQ_S] + a * jvs[636 * KQ_S];
      jvs[672 * KQ_S] = jvs[672 * KQ_S] + a * jvs[637 * KQ_S];
    }
    { const double a = -jvs[668 * KQ_S] / jvs[657 * KQ_S]; jvs[668 * KQ_S] = -a;
      jvs[669 * KQ_S] = jvs[669 * KQ_S] + a * jvs[658 * KQ_S];
      jvs[670 * KQ_S] = jvs[670 * KQ_S] + a * jvs[659 * KQ_S];
      jvs[671 * KQ_S] = jvs[671 * KQ_S] + a * jvs[660 * KQ_S];
      jvs[672 * KQ_S] = jvs[672 * KQ_S] + a * jvs[661 * KQ_S];
    }
    return 0;
}

KQ_HD KQ_NOINLINE int kqu_decomp_6(double* jvs)
{
    if (fabs(jvs[685 * KQ_S]) < DBL_MIN) return 159;
    { const double a = -jvs[673 * KQ_S] / jvs[214 * KQ_S]; jvs[673 * KQ_S] = -a;
      jvs[685 * KQ_S] = jvs[685 * KQ_S] + a * jvs[215 * KQ_S];
    }
    { const double a = -jvs[674 * KQ_S] / jvs[337 * KQ_S]; jvs[674 * KQ_S] = -a;
      jvs[679 * KQ_S] = jvs[679 * KQ_S] + a * jvs[338 * KQ_S];
      jvs[682 * KQ_S] = jvs[682 * KQ_S] + a * jvs[339 * KQ_S];
      jvs[687 * KQ_S] = jvs[687 * KQ_S] + a * jvs[340 * KQ_S];
    }
    { const double a = -jvs[675 * KQ_S] / jvs[446 * KQ_S]; jvs[675 * KQ_S] = -a;
      jvs[682 * KQ_S] = jvs[682 * KQ_S] + a * jvs[447 * KQ_S];
      jvs[683 * KQ_S] = jvs[683 * KQ_S] + a * jvs[448 * KQ_S];
      jvs[684 * KQ_S] = jvs[684 * KQ_S] + a * jvs[449 * KQ_S];
      jvs[685 * KQ_S] = jvs[685 * KQ_S] + a * jvs[450 * KQ_S];
    }
    { const double a = -jvs[676 * KQ_S] / jvs[462 * KQ_S]; jvs[676 * KQ_S] = -a;
      jvs[677 * KQ_S] = jvs[677 * KQ_S] + a * jvs[463 * KQ_S];
      jvs[679 * KQ_S] = jvs[679 * KQ_S] + a * jvs[464 * KQ_S];
      jvs[680 * KQ_S] = jvs[680 * KQ_S] + a * jvs[465 * KQ_S];
      jvs[682 * KQ_S] = jvs[682 * KQ_S] + a * jvs[466 * KQ_S];
      jvs[683 * KQ_S] = jvs[683 * KQ_S] + a * jvs[467 * KQ_S];
      jvs[684 * KQ_S] = jvs[684 * KQ_S] + a * jvs[468 * KQ_S];
    }
    { const double a = -jvs[677 * KQ_S] / jvs[488 * KQ_S]; jvs[677 * KQ_S] = -a;
      jvs[678 * KQ_S] = jvs[678 * KQ_S] + a * jvs[489 * KQ_S];
      jvs[681 * KQ_S] = jvs[681 * KQ_S] + a * jvs[490 * KQ_S];
      jvs[682 * KQ_S] = jvs[682 * KQ_S] + a * jvs[491 * KQ_S];
      jvs[683 * KQ_S] = jvs[683 * KQ_S] + a * jvs[492 * KQ_S];
      jvs[685 * KQ_S] = jvs[685 * KQ_S] + a * jvs[493 * KQ_S];
    }
    { const double a = -jvs[678 * KQ_S] / jvs[494 * KQ_S]; jvs[678 * KQ_S] = -a;
      jvs[681 * KQ_S] = jvs[681 * KQ_S] + a * jvs[495 * KQ_S];
      jvs[682 * KQ_S] = jvs[682 * KQ_S] + a * jvs[496 * KQ_S];
      jvs[684 * KQ_S] = jvs[684 * KQ_S] + a * jvs[497 * KQ_S];
      jvs[685 * KQ_S] = jvs[685 * KQ_S] + a * jvs[498 * KQ_S];
      jvs[687 * KQ_S] = jvs[687 * KQ_S] + a * jvs[499 * KQ_S];
    }
    { const double a = -jvs[679 * KQ_S] / jvs[505 * KQ_S]; jvs[679 * KQ_S] = -a;
      jvs[681 * KQ_S] = jvs[681 * KQ_S] + a * jvs[506 * KQ_S];
      jvs[682 * KQ_S] = jvs[682 * KQ_S] + a * jvs[507 * KQ_S];
      jvs[683 * KQ_S] = jvs[683 * KQ_S] + a * jvs[508 * KQ_S];
      jvs[684 * KQ_S] = jvs[684 * KQ_S] + a * jvs[509 * KQ_S];
      jvs[685 * KQ_S] = jvs[685 * KQ_S] + a * jvs[510 * KQ_S];
      jvs[686 * KQ_S] = jvs[686 * KQ_S] + a * jvs[511 * KQ_S];
      jvs[687 * KQ_S] = jvs[687 * KQ_S] + a * jvs[512 * KQ_S];
    }
    { const double a = -jvs[680 * KQ_S] / jvs[555 * KQ_S]; jvs[680 * KQ_S] = -a;
      jvs[681 * KQ_S] = jvs[681 * KQ_S] + a * jvs[556 * KQ_S];
      jvs[682 * KQ_S] = jvs[682 * KQ_S] + a * jvs[557 * KQ_S];
      jvs[683 * KQ_S] = jvs[683 * KQ_S] + a * jvs[558 * KQ_S];
      jvs[684 * KQ_S] = jvs[684 * KQ_S] + a * jvs[559 * KQ_S];
      jvs[685 * KQ_S] = jvs[685 * KQ_S] + a * jvs[560 * KQ_S];
      jvs[686 * KQ_S] = jvs[686 * KQ_S] + a * jvs[561 * KQ_S];
      jvs[687 * KQ_S] = jvs[687 * KQ_S] + a * jvs[562 * KQ_S];
    }
    { const double a = -jvs[681 * KQ_S] / jvs[584 * KQ_S]; jvs[681 * KQ_S] = -a;
      jvs[682 * KQ_S] = jvs[682 * KQ_S] + a * jvs[585 * KQ_S];
      jvs[683 * KQ_S] = jvs[683 * KQ_S] + a * jvs[586 * KQ_S];
      jvs[684 * KQ_S] = jvs[684 * KQ_S] + a * jvs[587 * KQ_S];
      jvs[685 * KQ_S] = jvs[685 * KQ_S] + a * jvs[588 * KQ_S];
      jvs[686 * KQ_S] = jvs[686 * KQ_S] + a * jvs[589 * KQ_S];
      jvs[687 * KQ_S] = jvs[687 * KQ_S] + a * jvs[590 * KQ_S];
    }
    { const double a = -jvs[682 * KQ_S] / jvs[632 * KQ_S]; jvs[682 * KQ_S] = -a;
      jvs[683 * KQ_S] = jvs[683 * KQ_S] + a * jvs[633 * KQ_S];
      jvs[684 * KQ_S] = jvs[684 * KQ_S] + a * jvs[634 * KQ_S];
      jvs[685 * KQ_S] = jvs[685 * KQ_S] + a * jvs[635 * KQ_S];
      jvs[686 * KQ_S] = jvs[686 * KQ_S] + a * jvs[636 * KQ_S];
      jvs[687 * KQ_S] = jvs[687 * KQ_S] + a * jvs[637 * KQ_S];
    }
    { const double a = -jvs[683 * KQ_S] / jvs[657 * KQ_S]; jvs[683 * KQ_S] = -a;
      jvs[684 * KQ_S] = jvs[684 * KQ_S] + a * jvs[658 * KQ_S];
      jvs[685 * KQ_S] = jvs[685 * KQ_S] + a * jvs[659 * KQ_S];
      jvs[686 * KQ_S] = jvs[686 * KQ_S] + a * jvs[660 * KQ_S];
      jvs[687 * KQ_S] = jvs[687 * KQ_S] + a * jvs[661 * KQ_S];
    }
    { const double a = -jvs[684 * KQ_S] / jvs[669 * KQ_S]; jvs[684 * KQ_S] = -a;
      jvs[685 * KQ_S] = jvs[685 * KQ_S] + a * jvs[670 * KQ_S];
      jvs[686 * KQ_S] = jvs[686 * KQ_S] + a * jvs[671 * KQ_S];
      jvs[687 * KQ_S] = jvs[687 * KQ_S] + a * jvs[672 * KQ_S];
    }
    if (fabs(jvs[700 * KQ_S]) < DBL_MIN) return 160;
    { const double a = -jvs[688 * KQ_S] / jvs[15 * KQ_S]; jvs[688 * KQ_S] = -a;
    }
    { const double a = -jvs[689 * KQ_S] / jvs[16 * KQ_S]; jvs[689 * KQ_S] = -a;
    }
    { const double a = -jvs[690 * KQ_S] / jvs[438 * KQ_S]; jvs[690 * KQ_S] = -a;
      jvs[691 * KQ_S] = jvs[691 * KQ_S] + a * jvs[439 * KQ_S];
      jvs[692 * KQ_S] = jvs[692 * KQ_S] + a * jvs[440 * KQ_S];
      jvs[697 * KQ_S] = jvs[697 * KQ_S] + a * jvs[441 * KQ_S];
      jvs[700 * KQ_S] = jvs[700 * KQ_S] + a * jvs[442 * KQ_S];
    }
    { const double a = -jvs[691 * KQ_S] / jvs[470 * KQ_S]; jvs[691 * KQ_S] = -a;
      jvs[692 * KQ_S] = jvs[692 * KQ_S] + a * jvs[471 * KQ_S];
      jvs[693 * KQ_S] = jvs[693 * KQ_S] + a * jvs[472 * KQ_S];
      jvs[697 * KQ_S] = jvs[697 * KQ_S] + a * jvs[473 * KQ_S];
      jvs[700 * KQ_S] = jvs[700 * KQ_S] + a * jvs[474 * KQ_S];
      jvs[701 * KQ_S] = jvs[701 * KQ_S] + a * jvs[475 * KQ_S];
    }
    { const double a = -jvs[692 * KQ_S] / jvs[480 * KQ_S]; jvs[692 * KQ_S] = -a;
      jvs[693 * KQ_S] = jvs[693 * KQ_S] + a * jvs[481 * KQ_S];
      jvs[696 * KQ_S] = jvs[696 * KQ_S] + a * jvs[482 * KQ_S];
      jvs[697 * KQ_S] = jvs[697 * KQ_S] + a * jvs[483 * KQ_S];
      jvs[700 * KQ_S] = jvs[700 * KQ_S] + a * jvs[484 * KQ_S];
      jvs[701 * KQ_S] = jvs[701 * KQ_S] + a * jvs[485 * KQ_S];
    }
    { const double a = -jvs[693 * KQ_S] / jvs[528 * KQ_S]; jvs[693 * KQ_S] = -a;
      jvs[694 * KQ_S] = jvs[694 * KQ_S] + a * jvs[529 * KQ_S];
      jvs[695 * KQ_S] = jvs[695 * KQ_S] + a * jvs[530 * KQ_S];
      jvs[696 * KQ_S] = jvs[696 * KQ_S] + a * jvs[531 * KQ_S];
      jvs[697 * KQ_S] = jvs[697 * KQ_S] + a * jvs[532 * KQ_S];
      jvs[698 * KQ_S] = jvs[698 * KQ_S] + a * jvs[533 * KQ_S];
      jvs[699 * KQ_S] = jvs[699 * KQ_S] + a * jvs[534 * KQ_S];
      jvs[700 * KQ_S] = jvs[700 * KQ_S] + a * jvs[535 * KQ_S];
      jvs[701 * KQ_S] = jvs[701 * KQ_S] + a * jvs[536 * KQ_S];
    }
    { const double a = -jvs[694 * KQ_S] / jvs[555 * KQ_S]; jvs[694 * KQ_S] = -a;
      jvs[695 * KQ_S] = jvs[695 * KQ_S] + a * jvs[556 * KQ_S];
      jvs[696 * KQ_S] = jvs[696 * KQ_S] + a * jvs[557 * KQ_S];
      jvs[697 * KQ_S] = jvs[697 * KQ_S] + a * jvs[558 * KQ_S];
      jvs[698 * KQ_S] = jvs[698 * KQ_S] + a * jvs[559 * KQ_S];
      jvs[699 * KQ_S] = jvs[699 * KQ_S] + a * jvs[560 * KQ_S];
      jvs[700 * KQ_S] = jvs[700 * KQ_S] + a * jvs[561 * KQ_S];
      jvs[701 * KQ_S] = jvs[701 * KQ_S] + a * jvs[562 * KQ_S];
    }
    { const double a = -jvs[695 * KQ_S] / jvs[584 * KQ_S]; jvs[695 * KQ_S] = -a;
      jvs[696 * KQ_S] = jvs[696 * KQ_S] + a * jvs[585 * KQ_S];
      jvs[697 * KQ_S] = jvs[697 * KQ_S] + a * jvs[586 * KQ_S];
      jvs[698 * KQ_S] = jvs[698 * KQ_S] + a * jvs[587 * KQ_S];
      jvs[699 * KQ_S] = jvs[699 * KQ_S] + a * jvs[588 * KQ_S];
      jvs[700 * KQ_S] = jvs[700 * KQ_S] + a * jvs[589 * KQ_S];
      jvs[701 * KQ_S] = jvs[701 * KQ_S] + a * jvs[590 * KQ_S];
    }
    { const double a = -jvs[696 * KQ_S] / jvs[632 * KQ_S]; jvs[696 * KQ_S] = -a;
      jvs[697 * KQ_S] = jvs[697 * KQ_S] + a * jvs[633 * KQ_S];
      jvs[698 * KQ_S] = jvs[698 * KQ_S] + a * jvs[634 * KQ_S];
      jvs[699 * KQ_S] = jvs[699 * KQ_S] + a * jvs[635 * KQ_S];
      jvs[700 * KQ_S] = jvs[700 * KQ_S] + a * jvs[636 * KQ_S];
      jvs[701 * KQ_S] = jvs[701 * KQ_S] + a * jvs[637 * KQ_S];
    }
    { const double a = -jvs[697 * KQ_S] / jvs[657 * KQ_S]; jvs[697 * KQ_S] = -a;
      jvs[698 * KQ_S] = jvs[698 * KQ_S] + a * jvs[658 * KQ_S];
      jvs[699 * KQ_S] = jvs[699 * KQ_S] + a * jvs[659 * KQ_S];
      jvs[700 * KQ_S] = jvs[700 * KQ_S] + a * jvs[660 * KQ_S];
      jvs[701 * KQ_S] = jvs[701 * KQ_S] + a * jvs[661 * KQ_S];
    }
    { const double a = -jvs[698 * KQ_S] / jvs[669 * KQ_S]; jvs[698 * KQ_S] = -a;
      jvs[699 * KQ_S] = jvs[699 * KQ_S] + a * jvs[670 * KQ_S];
      jvs[700 * KQ_S] = jvs[700 * KQ_S] + a * jvs[671 * KQ_S];
      jvs[701 * KQ_S] = jvs[701 * KQ_S] + a * jvs[672 * KQ_S];
    }
    { const double a = -jvs[699 * KQ_S] / jvs[685 * KQ_S]; jvs[699 * KQ_S] = -a;
      jvs[700 * KQ_S] = jvs[700 * KQ_S] + a * jvs[686 * KQ_S];
      jvs[701 * KQ_S] = jvs[701 * KQ_S] + a * jvs[687 * KQ_S];
    }
    return 0;
}

KQ_HD KQ_NOINLINE int kqu_decomp_7(double* jvs)
{
    if (fabs(jvs[737 * KQ_S]) < DBL_MIN) return 161;
    { const double a = -jvs[702 * KQ_S] / jvs[237 * KQ_S]; jvs[702 * KQ_S] = -a;
      jvs[737 * KQ_S] = jvs[737 * KQ_S] + a * jvs[238 * KQ_S];
    }
    { const double a = -jvs[703 * KQ_S] / jvs[241 * KQ_S]; jvs[703 * KQ_S] = -a;
      jvs[737 * KQ_S] = jvs[737 * KQ_S] + a * jvs[242 * KQ_S];
    }
    { const double a = -jvs[704 * KQ_S] / jvs[267 * KQ_S]; jvs[704 * KQ_S] = -a;
      jvs[737 * KQ_S] = jvs[737 * KQ_S] + a * jvs[268 * KQ_S];
    }
    { const double a = -jvs[705 * KQ_S] / jvs[313 * KQ_S]; jvs[705 * KQ_S] = -a;
      jvs[707 * KQ_S] = jvs[707 * KQ_S] + a * jvs[314 * KQ_S];
      jvs[721 * KQ_S] = jvs[721 * KQ_S] + a * jvs[315 * KQ_S];
      jvs[730 * KQ_S] = jvs[730 * KQ_S] + a * jvs[316 * KQ_S];
    }
    { const double a = -jvs[706 * KQ_S] / jvs[337 * KQ_S]; jvs[706 * KQ_S] = -a;
      jvs[728 * KQ_S] = jvs[728 * KQ_S] + a * jvs[338 * KQ_S];
      jvs[732 * KQ_S] = jvs[732 * KQ_S] + a * jvs[339 * KQ_S];
      jvs[737 * KQ_S] = jvs[737 * KQ_S] + a * jvs[340 * KQ_S];
    }
    { const double a = -jvs[707 * KQ_S] / jvs[342 * KQ_S]; jvs[707 * KQ_S] = -a;
      jvs[730 * KQ_S] = jvs[730 * KQ_S] + a * jvs[343 * KQ_S];
      jvs[733 * KQ_S] = jvs[733 * KQ_S] + a * jvs[344 * KQ_S];
    }
    { const double a = -jvs[708 * KQ_S] / jvs[350 * KQ_S]; jvs[708 * KQ_S] = -a;
      jvs[710 * KQ_S] = jvs[710 * KQ_S] + a * jvs[351 * KQ_S];
      jvs[715 * KQ_S] = jvs[715 * KQ_S] + a * jvs[352 * KQ_S];
      jvs[732 * KQ_S] = jvs[732 * KQ_S] + a * jvs[353 * KQ_S];
      jvs[737 * KQ_S] = jvs[737 * KQ_S] + a * jvs[354 * KQ_S];
    }
    { const double a = -jvs[709 * KQ_S] / jvs[360 * KQ_S]; jvs[709 * KQ_S] = -a;
      jvs[710 * KQ_S] = jvs[710 * KQ_S] + a * jvs[361 * KQ_S];
      jvs[732 * KQ_S] = jvs[732 * KQ_S] + a * jvs[362 * KQ_S];
      jvs[737 * KQ_S] = jvs[737 * KQ_S] + a * jvs[363 * KQ_S];
    }
    { const double a = -jvs[710 * KQ_S] / jvs[366 * KQ_S]; jvs[710 * KQ_S] = -a;
      jvs[715 * KQ_S] = jvs[715 * KQ_S] + a * jvs[367 * KQ_S];
      jvs[719 * KQ_S] = jvs[719 * KQ_S] + a * jvs[368 * KQ_S];
      jvs[732 * KQ_S] = jvs[732 * KQ_S] + a * jvs[369 * KQ_S];
      jvs[737 * KQ_S] = jvs[737 * KQ_S] + a * jvs[370 * KQ_S];
    }
    { const double a = -jvs[711 * KQ_S] / jvs[372 * KQ_S]; jvs[711 * KQ_S] = -a;
      jvs[712 * KQ_S] = jvs[712 * KQ_S] + a * jvs[373 * KQ_S];
      jvs[732 * KQ_S] = jvs[732 * KQ_S] + a * jvs[374 * KQ_S];
      jvs[737 * KQ_S] = jvs[737 * KQ_S] + a * jvs[375 * KQ_S];
    }
    { const double a = -jvs[712 * KQ_S] / jvs[378 * KQ_S]; jvs[712 * KQ_S] = -a;
      jvs[732 * KQ_S] = jvs[732 * KQ_S] + a * jvs[379 * KQ_S];
      jvs[737 * KQ_S] = jvs[737 * KQ_S] + a * jvs[380 * KQ_S];
    }
    { const double a = -jvs[713 * KQ_S] / jvs[383 * KQ_S]; jvs[713 * KQ_S] = -a;
      jvs[714 * KQ_S] = jvs[714 * KQ_S] + a * jvs[384 * KQ_S];
      jvs[732 * KQ_S] = jvs[732 * KQ_S] + a * jvs[385 * KQ_S];
      jvs[737 * KQ_S] = jvs[737 * KQ_S] + a * jvs[386 * KQ_S];
    }
    { const double a = -jvs[714 * KQ_S] / jvs[390 * KQ_S]; jvs[714 * KQ_S] = -a;
      jvs[732 * KQ_S] = jvs[732 * KQ_S] + a * jvs[391 * KQ_S];
      jvs[737 * KQ_S] = jvs[737 * KQ_S] + a * jvs[392 * KQ_S];
    }
    { const double a = -jvs[715 * KQ_S] / jvs[396 * KQ_S]; jvs[715 * KQ_S] = -a;
      jvs[719 * KQ_S] = jvs[719 * KQ_S] + a * jvs[397 * KQ_S];
      jvs[732 * KQ_S] = jvs[732 * KQ_S] + a * jvs[398 * KQ_S];
      jvs[737 * KQ_S] = jvs[737 * KQ_S] + a * jvs[399 * KQ_S];
    }
    { const double a = -jvs[716 * KQ_S] / jvs[400 * KQ_S]; jvs[716 * KQ_S] = -a;
      jvs[720 * KQ_S] = jvs[720 * KQ_S] + a * jvs[401 * KQ_S];
      jvs[732 * KQ_S] = jvs[732 * KQ_S] + a * jvs[402 * KQ_S];
      jvs[737 * KQ_S] = jvs[737 * KQ_S] + a * jvs[403 * KQ_S];
    }
    { const double a = -jvs[717 * KQ_S] / jvs[405 * KQ_S]; jvs[717 * KQ_S] = -a;
      jvs[718 * KQ_S] = jvs[718 * KQ_S] + a * jvs[406 * KQ_S];
      jvs[732 * KQ_S] = jvs[732 * KQ_S] + a * jvs[407 * KQ_S];
      jvs[737 * KQ_S] = jvs[737 * KQ_S] + a * jvs[408 * KQ_S];
    }
    { const double a = -jvs[718 * KQ_S] / jvs[410 * KQ_S]; jvs[718 * KQ_S] = -a;
      jvs[732 * KQ_S] = jvs[732 * KQ_S] + a * jvs[411 * KQ_S];
      jvs[737 * KQ_S] = jvs[737 * KQ_S] + a * jvs[412 * KQ_S];
    }
    { const double a = -jvs[719 * KQ_S] / jvs[418 * KQ_S]; jvs[719 * KQ_S] = -a;
      jvs[732 * KQ_S] = jvs[732 * KQ_S] + a * jvs[419 * KQ_S];
      jvs[737 * KQ_S] = jvs[737 * KQ_S] + a * jvs[420 * KQ_S];
    }
    { const double a = -jvs[720 * KQ_S] / jvs[423 * KQ_S]; jvs[720 * KQ_S] = -a;
      jvs[724 * KQ_S] = jvs[724 * KQ_S] + a * jvs[424 * KQ_S];
      jvs[725 * KQ_S] = jvs[725 * KQ_S] + a * jvs[425 * KQ_S];
      jvs[732 * KQ_S] = jvs[732 * KQ_S] + a * jvs[426 * KQ_S];
      jvs[737 * KQ_S] = jvs[737 * KQ_S] + a * jvs[427 * KQ_S];
    }
    { const double a = -jvs[721 * KQ_S] / jvs[431 * KQ_S]; jvs[721 * KQ_S] = -a;
      jvs[730 * KQ_S] = jvs[730 * KQ_S] + a * jvs[432 * KQ_S];
      jvs[731 * KQ_S] = jvs[731 * KQ_S] + a * jvs[433 * KQ_S];
      jvs[733 * KQ_S] = jvs[733 * KQ_S] + a * jvs[434 * KQ_S];
      jvs[737 * KQ_S] = jvs[737 * KQ_S] + a * jvs[435 * KQ_S];
    }
    { const double a = -jvs[722 * KQ_S] / jvs[452 * KQ_S]; jvs[722 * KQ_S] = -a;
      jvs[727 * KQ_S] = jvs[727 * KQ_S] + a * jvs[453 * KQ_S];
      jvs[731 * KQ_S] = jvs[731 * KQ_S] + a * jvs[454 * KQ_S];
      jvs[732 * KQ_S] = jvs[732 * KQ_S] + a * jvs[455 * KQ_S];
      jvs[733 * KQ_S] = jvs[733 * KQ_S] + a * jvs[456 * KQ_S];
      jvs[737 * KQ_S] = jvs[737 * KQ_S] + a * jvs[457 * KQ_S];
    }
    { const double a = -jvs[723 * KQ_S] / jvs[462 * KQ_S]; jvs[723 * KQ_S] = -a;
      jvs[726 * KQ_S] = jvs[726 * KQ_S] + a * jvs[463 * KQ_S];
      jvs[728 * KQ_S] = jvs[728 * KQ_S] + a * jvs[464 * KQ_S];
      jvs[730 * KQ_S] = jvs[730 * KQ_S] + a * jvs[465 * KQ_S];
      jvs[732 * KQ_S] = jvs[732 * KQ_S] + a * jvs[466 * KQ_S];
      jvs[733 * KQ_S] = jvs[733 * KQ_S] + a * jvs[467 * KQ_S];
      jvs[734 * KQ_S] = jvs[734 * KQ_S] + a * jvs[468 * KQ_S];
    }
    { const double a = -jvs[724 * KQ_S] / jvs[470 * KQ_S]; jvs[724 * KQ_S] = -a;
      jvs[725 * KQ_S] = jvs[725 * KQ_S] + a * jvs[471 * KQ_S];
      jvs[729 * KQ_S] = jvs[729 * KQ_S] + a * jvs[472 * KQ_S];
      jvs[733 * KQ_S] = jvs[733 * KQ_S] + a * jvs[473 * KQ_S];
      jvs[736 * KQ_S] = jvs[736 * KQ_S] + a * jvs[474 * KQ_S];
      jvs[737 * KQ_S] = jvs[737 * KQ_S] + a * jvs[475 * KQ_S];
    }
    { const double a = -jvs[725 * KQ_S] / jvs[480 * KQ_S]; jvs[725 * KQ_S] = -a;
      jvs[729 * KQ_S] = jvs[729 * KQ_S] + a * jvs[481 * KQ_S];
      jvs[732 * KQ_S] = jvs[732 * KQ_S] + a * jvs[482 * KQ_S];
      jvs[733 * KQ_S] = jvs[733 * KQ_S] + a * jvs[483 * KQ_S];
      jvs[736 * KQ_S] = jvs[736 * KQ_S] + a * jvs[484 * KQ_S];
      jvs[737 * KQ_S] = jvs[737 * KQ_S] + a * jvs[485 * KQ_S];
    }
    { const double a = -jvs[726 * KQ_S] / jvs[488 * KQ_S]; jvs[726 * KQ_S] = -a;
      jvs[727 * KQ_S] = jvs[727 * KQ_S] + a * jvs[489 * KQ_S];
      jvs[731 * KQ_S] = jvs[731 * KQ_S] + a * jvs[490 * KQ_S];
      jvs[732 * KQ_S] = jvs[732 * KQ_S] + a * jvs[491 * KQ_S];
      jvs[733 * KQ_S] = jvs[733 * KQ_S] + a * jvs[492 * KQ_S];
      jvs[735 * KQ_S] = jvs[735 * KQ_S] + a * jvs[493 * KQ_S];
    }
    { const double a = -jvs[727 * KQ_S] / jvs[494 * KQ_S]; jvs[727 * KQ_S] = -a;
      jvs[731 * KQ_S] = jvs[731 * KQ_S] + a * jvs[495 * KQ_S];
      jvs[732 * KQ_S] = jvs[732 * KQ_S] + a * jvs[496 * KQ_S];
      jvs[734 * KQ_S] = jvs[734 * KQ_S] + a * jvs[497 * KQ_S];
      jvs[735 * KQ_S] = jvs[735 * KQ_S] + a * jvs[498 * KQ_S];
      jvs[737 * KQ_S] = jvs[737 * KQ_S] + a * jvs[499 * KQ_S];
    }
    { const double a = -jvs[728 * KQ_S] / jvs[505 * KQ_S]; jvs[728 * KQ_S] = -a;
      jvs[731 * KQ_S] = jvs[731 * KQ_S] + a * jvs[506 * KQ_S];
      jvs[732 * KQ_S] = jvs[732 * KQ_S] + a * jvs[507 * KQ_S];
      jvs[733 * KQ_S] = jvs[733 * KQ_S] + a * jvs[508 * KQ_S];
      jvs[734 * KQ_S] = jvs[734 * KQ_S] + a * jvs[509 * KQ_S];
      jvs[735 * KQ_S] = jvs[735 * KQ_S] + a * jvs[510 * KQ_S];
      jvs[736 * KQ_S] = jvs[736 * KQ_S] + a * jvs[511 * KQ_S];
      jvs[737 * KQ_S] = jvs[737 * KQ_S] + a * jvs[512 * KQ_S];
    }
    { const double a = -jvs[729 * KQ_S] / jvs[528 * KQ_S]; jvs[729 * KQ_S] = -a;
      jvs[730 * KQ_S] = jvs[730 * KQ_S] + a * jvs[529 * KQ_S];
      jvs[731 * KQ_S] = jvs[731 * KQ_S] + a * jvs[530 * KQ_S];
      jvs[732 * KQ_S] = jvs[732 * KQ_S] + a * jvs[531 * KQ_S];
      jvs[733 * KQ_S] = jvs[733 * KQ_S] + a * jvs[532 * KQ_S];
      jvs[734 * KQ_S] = jvs[734 * KQ_S] + a * jvs[533 * KQ_S];
      jvs[735 * KQ_S] = jvs[735 * KQ_S] + a * jvs[534 * KQ_S];
      jvs[736 * KQ_S] = jvs[736 * KQ_S] + a * jvs[535 * KQ_S];
      jvs[737 * KQ_S] = jvs[737 * KQ_S] + a * jvs[536 * KQ_S];
    }
    { const double a = -jvs[730 * KQ_S] / jvs[555 * KQ_S]; jvs[730 * KQ_S] = -a;
      jvs[731 * KQ_S] = jvs[731 * KQ_S] + a * jvs[556 * KQ_S];
      jvs[732 * KQ_S] = jvs[732 * KQ_S] + a * jvs[557 * KQ_S];
      jvs[733 * KQ_S] = jvs[733 * KQ_S] + a * jvs[558 * KQ_S];
      jvs[734 * KQ_S] = jvs[734 * KQ_S] + a * jvs[559 * KQ_S];
      jvs[735 * KQ_S] = jvs[735 * KQ_S] + a * jvs[560 * KQ_S];
      jvs[736 * KQ_S] = jvs[736 * KQ_S] + a * jvs[561 * KQ_S];
      jvs[737 * KQ_S] = jvs[737 * KQ_S] + a * jvs[562 * KQ_S];
    }
    { const double a = -jvs[731 * KQ_S] / jvs[584 * KQ_S]; jvs[731 * KQ_S] = -a;
      jvs[732 * KQ_S] = jvs[732 * KQ_S] + a * jvs[585 * KQ_S];
      jvs[733 * KQ_S] = jvs[733 * KQ_S] + a * jvs[586 * KQ_S];
      jvs[734 * KQ_S] = jvs[734 * KQ_S] + a * jvs[587 * KQ_S];
      jvs[735 * KQ_S] = jvs[735 * KQ_S] + a * jvs[588 * KQ_S];
      jvs[736 * KQ_S] = jvs[736 * KQ_S] + a * jvs[589 * KQ_S];
      jvs[737 * KQ_S] = jvs[737 * KQ_S] + a * jvs[590 * KQ_S];
    }
    { const double a = -jvs[732 * KQ_S] / jvs[632 * KQ_S]; jvs[732 * KQ_S] = -a;
      jvs[733 * KQ_S] = jvs[733 * KQ_S] + a * jvs[633 * KQ_S];
      jvs[734 * KQ_S] = jvs[734 * KQ_S] + a * jvs[634 * KQ_S];
      jvs[735 * KQ_S] = jvs[735 * KQ_S] + a * jvs[635 * KQ_S];
      jvs[736 * KQ_S] = jvs[736 * KQ_S] + a * jvs[636 * KQ_S];
      jvs[737 * KQ_S] = jvs[737 * KQ_S] + a * jvs[637 * KQ_S];
    }
    { const double a = -jvs[733 * KQ_S] / jvs[657 * KQ_S]; jvs[733 * KQ_S] = -a;
      jvs[734 * KQ_S] = jvs[734 * KQ_S] + a * jvs[658 * KQ_S];
      jvs[735 * KQ_S] = jvs[735 * KQ_S] + a * jvs[659 * KQ_S];
      jvs[736 * KQ_S] = jvs[736 * KQ_S] + a * jvs[660 * KQ_S];
      jvs[737 * KQ_S] = jvs[737 * KQ_S] + a * jvs[661 * KQ_S];
    }
    { const double a = -jvs[734 * KQ_S] / jvs[669 * KQ_S]; jvs[734 * KQ_S] = -a;
      jvs[735 * KQ_S] = jvs[735 * KQ_S] + a * jvs[670 * KQ_S];
      jvs[736 * KQ_S] = jvs[736 * KQ_S] + a * jvs[671 * KQ_S];
      jvs[737 * KQ_S] = jvs[737 * KQ_S] + a * jvs[672 * KQ_S];
    }
    { const double a = -jvs[735 * KQ_S] / jvs[685 * KQ_S]; jvs[735 * KQ_S] = -a;
      jvs[736 * KQ_S] = jvs[736 * KQ_S] + a * jvs[686 * KQ_S];
      jvs[737 * KQ_S] = jvs[737 * KQ_S] + a * jvs[687 * KQ_S];
    }
    { const double a = -jvs[736 * KQ_S] / jvs[700 * KQ_S]; jvs[736 * KQ_S] = -a;
      jvs[737 * KQ_S] = jvs[737 * KQ_S] + a * jvs[701 * KQ_S];
    }
    return 0;
}

KQ_HD inline int kqu_decomp(double* jvs)
{
    int rc;
    if ((rc = kqu_decomp_0(jvs)) != 0) return rc;
    if ((rc = kqu_decomp_1(jvs)) != 0) return rc;
    if ((rc = kqu_decomp_2(jvs)) != 0) return rc;
    if ((rc = kqu_decomp_3(jvs)) != 0) return rc;
    if ((rc = kqu_decomp_4(jvs)) != 0) return rc;
    if ((rc = kqu_decomp_5(jvs)) != 0) return rc;
    if ((rc = kqu_decomp_6(jvs)) != 0) return rc;
    if ((rc = kqu_decomp_7(jvs)) != 0) return rc;
    return 0;
}

KQ_HD KQ_NOINLINE void kqu_solve_f0(const double* jvs, double* x)
{
    x[8 * KQ_S] = x[8 * KQ_S] - jvs[8 * KQ_S] * x[7 * KQ_S];
    x[9 * KQ_S] = x[9 * KQ_S] - jvs[10 * KQ_S] * x[5 * KQ_S];
    x[11 * KQ_S] = x[11 * KQ_S] - jvs[13 * KQ_S] * x[6 * KQ_S];
    x[17 * KQ_S] = x[17 * KQ_S] - jvs[20 * KQ_S] * x[3 * KQ_S];
    x[36 * KQ_S] = x[36 * KQ_S] - jvs[73 * KQ_S] * x[8 * KQ_S];
    x[37 * KQ_S] = x[37 * KQ_S] - jvs[75 * KQ_S] * x[12 * KQ_S];
    x[38 * KQ_S] = x[38 * KQ_S] - jvs[77 * KQ_S] * x[13 * KQ_S];
    x[39 * KQ_S] = x[39 * KQ_S] - jvs[79 * KQ_S] * x[9 * KQ_S];
    x[40 * KQ_S] = x[40 * KQ_S] - jvs[81 * KQ_S] * x[10 * KQ_S];
    x[41 * KQ_S] = x[41 * KQ_S] - jvs[83 * KQ_S] * x[11 * KQ_S];
    x[43 * KQ_S] = x[43 * KQ_S] - jvs[87 * KQ_S] * x[14 * KQ_S];
    x[44 * KQ_S] = x[44 * KQ_S] - jvs[89 * KQ_S] * x[15 * KQ_S];
    x[45 * KQ_S] = x[45 * KQ_S] - jvs[91 * KQ_S] * x[16 * KQ_S];
    x[46 * KQ_S] = x[46 * KQ_S] - jvs[93 * KQ_S] * x[17 * KQ_S];
    x[75 * KQ_S] = x[75 * KQ_S] - jvs[172 * KQ_S] * x[74 * KQ_S];
    x[77 * KQ_S] = x[77 * KQ_S] - jvs[177 * KQ_S] * x[76 * KQ_S];
    x[104 * KQ_S] = x[104 * KQ_S] - jvs[236 * KQ_S] * x[78 * KQ_S];
    x[105 * KQ_S] = x[105 * KQ_S] - jvs[239 * KQ_S] * x[93 * KQ_S] - jvs[240 * KQ_S] * x[104 * KQ_S];
    x[106 * KQ_S] = x[106 * KQ_S] - jvs[243 * KQ_S] * x[85 * KQ_S];
    x[107 * KQ_S] = x[107 * KQ_S] - jvs[247 * KQ_S] * x[87 * KQ_S];
    x[108 * KQ_S] = x[108 * KQ_S] - jvs[251 * KQ_S] * x[1 * KQ_S] - jvs[252 * KQ_S] * x[107 * KQ_S];
    x[110 * KQ_S] = x[110 * KQ_S] - jvs[258 * KQ_S] * x[92 * KQ_S];
    x[111 * KQ_S] = x[111 * KQ_S] - jvs[262 * KQ_S] * x[2 * KQ_S] - jvs[263 * KQ_S] * x[110 * KQ_S];
    x[112 * KQ_S] = x[112 * KQ_S] - jvs[266 * KQ_S] * x[94 * KQ_S];
    x[114 * KQ_S] = x[114 * KQ_S] - jvs[272 * KQ_S] * x[113 * KQ_S];
    x[115 * KQ_S] = x[115 * KQ_S] - jvs[276 * KQ_S] * x[100 * KQ_S] - jvs[277 * KQ_S] * x[101 * KQ_S] - jvs[278 * KQ_S] * x[102 * KQ_S];
    x[118 * KQ_S] = x[118 * KQ_S] - jvs[293 * KQ_S] * x[83 * KQ_S] - jvs[294 * KQ_S] * x[116 * KQ_S] - jvs[295 * KQ_S] * x[117 * KQ_S];
    x[119 * KQ_S] = x[119 * KQ_S] - jvs[301 * KQ_S] * x[98 * KQ_S];
    x[120 * KQ_S] = x[120 * KQ_S] - jvs[304 * KQ_S] * x[90 * KQ_S] - jvs[305 * KQ_S] * x[119 * KQ_S];
    x[121 * KQ_S] = x[121 * KQ_S] - jvs[309 * KQ_S] * x[91 * KQ_S];
    x[123 * KQ_S] = x[123 * KQ_S] - jvs[317 * KQ_S] * x[109 * KQ_S] - jvs[318 * KQ_S] * x[122 * KQ_S];
    x[124 * KQ_S] = x[124 * KQ_S] - jvs[324 * KQ_S] * x[86 * KQ_S] - jvs[325 * KQ_S] * x[114 * KQ_S];
    x[125 * KQ_S] = x[125 * KQ_S] - jvs[336 * KQ_S] * x[73 * KQ_S];
    x[126 * KQ_S] = x[126 * KQ_S] - jvs[341 * KQ_S] * x[97 * KQ_S];
    x[131 * KQ_S] = x[131 * KQ_S] - jvs[364 * KQ_S] * x[128 * KQ_S] - jvs[365 * KQ_S] * x[130 * KQ_S];
    x[132 * KQ_S] = x[132 * KQ_S] - jvs[371 * KQ_S] * x[112 * KQ_S];
    x[133 * KQ_S] = x[133 * KQ_S] - jvs[376 * KQ_S] * x[82 * KQ_S] - jvs[377 * KQ_S] * x[132 * KQ_S];
    x[134 * KQ_S] = x[134 * KQ_S] - jvs[381 * KQ_S] * x[79 * KQ_S] - jvs[382 * KQ_S] * x[133 * KQ_S];
    x[135 * KQ_S] = x[135 * KQ_S] - jvs[387 * KQ_S] * x[132 * KQ_S] - jvs[388 * KQ_S] * x[133 * KQ_S] - jvs[389 * KQ_S] * x[134 * KQ_S];
    x[136 * KQ_S] = x[136 * KQ_S] - jvs[393 * KQ_S] * x[105 * KQ_S] - jvs[394 * KQ_S] * x[134 * KQ_S] - jvs[395 * KQ_S] * x[135 * KQ_S];
    x[138 * KQ_S] = x[138 * KQ_S] - jvs[404 * KQ_S] * x[104 * KQ_S];
    x[139 * KQ_S] = x[139 * KQ_S] - jvs[409 * KQ_S] * x[138 * KQ_S];
}

KQ_HD KQ_NOINLINE void kqu_solve_f1(const double* jvs, double* x)
{
    x[140 * KQ_S] = x[140 * KQ_S] - jvs[413 * KQ_S] * x[112 * KQ_S] - jvs[414 * KQ_S] * x[135 * KQ_S] - jvs[415 * KQ_S] * x[136 * KQ_S] - jvs[416 * KQ_S] * x[138 * KQ_S] - jvs[417 * KQ_S] * x[139 * KQ_S];
    x[141 * KQ_S] = x[141 * KQ_S] - jvs[421 * KQ_S] * x[89 * KQ_S] - jvs[422 * KQ_S] * x[137 * KQ_S];
    x[142 * KQ_S] = x[142 * KQ_S] - jvs[428 * KQ_S] * x[103 * KQ_S] - jvs[429 * KQ_S] * x[119 * KQ_S] - jvs[430 * KQ_S] * x[126 * KQ_S];
    x[143 * KQ_S] = x[143 * KQ_S] - jvs[436 * KQ_S] * x[80 * KQ_S] - jvs[437 * KQ_S] * x[119 * KQ_S];
    x[144 * KQ_S] = x[144 * KQ_S] - jvs[443 * KQ_S] * x[12 * KQ_S] - jvs[444 * KQ_S] * x[13 * KQ_S] - jvs[445 * KQ_S] * x[99 * KQ_S];
    x[145 * KQ_S] = x[145 * KQ_S] - jvs[451 * KQ_S] * x[84 * KQ_S];
    x[146 * KQ_S] = x[146 * KQ_S] - jvs[458 * KQ_S] * x[0 * KQ_S] - jvs[459 * KQ_S] * x[106 * KQ_S] - jvs[460 * KQ_S] * x[115 * KQ_S] - jvs[461 * KQ_S] * x[126 * KQ_S];
    x[147 * KQ_S] = x[147 * KQ_S] - jvs[469 * KQ_S] * x[143 * KQ_S];
    x[148 * KQ_S] = x[148 * KQ_S] - jvs[476 * KQ_S] * x[134 * KQ_S] - jvs[477 * KQ_S] * x[135 * KQ_S] - jvs[478 * KQ_S] * x[143 * KQ_S] - jvs[479 * KQ_S] * x[147 * KQ_S];
    x[149 * KQ_S] = x[149 * KQ_S] - jvs[486 * KQ_S] * x[96 * KQ_S] - jvs[487 * KQ_S] * x[129 * KQ_S];
    x[151 * KQ_S] = x[151 * KQ_S] - jvs[500 * KQ_S] * x[125 * KQ_S] - jvs[501 * KQ_S] * x[129 * KQ_S] - jvs[502 * KQ_S] * x[144 * KQ_S] - jvs[503 * KQ_S] * x[149 * KQ_S] - jvs[504 * KQ_S] * x[150 * KQ_S];
    x[152 * KQ_S] = x[152 * KQ_S] - jvs[513 * KQ_S] * x[107 * KQ_S] - jvs[514 * KQ_S] * x[108 * KQ_S] - jvs[515 * KQ_S] * x[130 * KQ_S] - jvs[516 * KQ_S] * x[131 * KQ_S] - jvs[517 * KQ_S] * x[136 * KQ_S] - jvs[518 * KQ_S] * x[137 * KQ_S] - jvs[519 * KQ_S] * x[140 * KQ_S] - jvs[520 * KQ_S] * x[141 * KQ_S] - jvs[521 * KQ_S] * x[143 * KQ_S] - jvs[522 * KQ_S] * x[146 * KQ_S] - jvs[523 * KQ_S] * x[147 * KQ_S] - jvs[524 * KQ_S] * x[148 * KQ_S] - jvs[525 * KQ_S] * x[149 * KQ_S] - jvs[526 * KQ_S] * x[150 * KQ_S] - jvs[527 * KQ_S] * x[151 * KQ_S];
    x[153 * KQ_S] = x[153 * KQ_S] - jvs[537 * KQ_S] * x[4 * KQ_S] - jvs[538 * KQ_S] * x[12 * KQ_S] - jvs[539 * KQ_S] * x[13 * KQ_S] - jvs[540 * KQ_S] * x[75 * KQ_S] - jvs[541 * KQ_S] * x[77 * KQ_S] - jvs[542 * KQ_S] * x[115 * KQ_S] - jvs[543 * KQ_S] * x[120 * KQ_S] - jvs[544 * KQ_S] * x[121 * KQ_S] - jvs[545 * KQ_S] * x[123 * KQ_S] - jvs[546 * KQ_S] * x[126 * KQ_S] - jvs[547 * KQ_S] * x[127 * KQ_S] - jvs[548 * KQ_S] * x[142 * KQ_S] - jvs[549 * KQ_S] * x[144 * KQ_S] - jvs[550 * KQ_S] * x[145 * KQ_S] - jvs[551 * KQ_S] * x[146 * KQ_S] - jvs[552 * KQ_S] * x[149 * KQ_S] - jvs[553 * KQ_S] * x[150 * KQ_S] - jvs[554 * KQ_S] * x[151 * KQ_S];
    x[154 * KQ_S] = x[154 * KQ_S] - jvs[563 * KQ_S] * x[81 * KQ_S] - jvs[564 * KQ_S] * x[104 * KQ_S] - jvs[565 * KQ_S] * x[105 * KQ_S] - jvs[566 * KQ_S] * x[112 * KQ_S] - jvs[567 * KQ_S] * x[119 * KQ_S] - jvs[568 * KQ_S] * x[132 * KQ_S] - jvs[569 * KQ_S] * x[133 * KQ_S] - jvs[570 * KQ_S] * x[136 * KQ_S] - jvs[571 * KQ_S] * x[137 * KQ_S] - jvs[572 * KQ_S] * x[138 * KQ_S] - jvs[573 * KQ_S] * x[139 * KQ_S] - jvs[574 * KQ_S] * x[140 * KQ_S] - jvs[575 * KQ_S] * x[141 * KQ_S] - jvs[576 * KQ_S] * x[142 * KQ_S] - jvs[577 * KQ_S] * x[145 * KQ_S] - jvs[578 * KQ_S] * x[147 * KQ_S] - jvs[579 * KQ_S] * x[148 * KQ_S] - jvs[580 * KQ_S] * x[149 * KQ_S] - jvs[581 * KQ_S] * x[150 * KQ_S] - jvs[582 * KQ_S] * x[152 * KQ_S] - jvs[583 * KQ_S] * x[153 * KQ_S];
    x[155 * KQ_S] = x[155 * KQ_S] - jvs[591 * KQ_S] * x[12 * KQ_S] - jvs[592 * KQ_S] * x[13 * KQ_S] - jvs[593 * KQ_S] * x[106 * KQ_S] - jvs[594 * KQ_S] * x[109 * KQ_S] - jvs[595 * KQ_S] * x[110 * KQ_S] - jvs[596 * KQ_S] * x[111 * KQ_S] - jvs[597 * KQ_S] * x[113 * KQ_S] - jvs[598 * KQ_S] * x[114 * KQ_S] - jvs[599 * KQ_S] * x[120 * KQ_S] - jvs[600 * KQ_S] * x[121 * KQ_S] - jvs[601 * KQ_S] * x[123 * KQ_S] - jvs[602 * KQ_S] * x[124 * KQ_S] - jvs[603 * KQ_S] * x[125 * KQ_S] - jvs[604 * KQ_S] * x[126 * KQ_S] - jvs[605 * KQ_S] * x[127 * KQ_S] - jvs[606 * KQ_S] * x[128 * KQ_S] - jvs[607 * KQ_S] * x[129 * KQ_S] - jvs[608 * KQ_S] * x[130 * KQ_S] - jvs[609 * KQ_S] * x[131 * KQ_S] - jvs[610 * KQ_S] * x[132 * KQ_S] - jvs[611 * KQ_S] * x[133 * KQ_S] - jvs[612 * KQ_S] * x[134 * KQ_S] - jvs[613 * KQ_S] * x[135 * KQ_S] - jvs[614 * KQ_S] * x[136 * KQ_S] - jvs[615 * KQ_S] * x[137 * KQ_S] - jvs[616 * KQ_S] * x[138 * KQ_S] - jvs[617 * KQ_S] * x[139 * KQ_S] - jvs[618 * KQ_S] * x[140 * KQ_S] - jvs[619 * KQ_S] * x[141 * KQ_S] - jvs[620 * KQ_S] * x[142 * KQ_S] - jvs[621 * KQ_S] * x[144 * KQ_S] - jvs[622 * KQ_S] * x[145 * KQ_S] - jvs[623 * KQ_S] * x[146 * KQ_S] - jvs[624 * KQ_S] * x[147 * KQ_S] - jvs[625 * KQ_S] * x[148 * KQ_S] - jvs[626 * KQ_S] * x[149 * KQ_S] - jvs[627 * KQ_S] * x[150 * KQ_S] - jvs[628 * KQ_S] * x[151 * KQ_S] - jvs[629 * KQ_S] * x[152 * KQ_S] - jvs[630 * KQ_S] * x[153 * KQ_S] - jvs[631 * KQ_S] * x[154 * KQ_S];
    x[156 * KQ_S] = x[156 * KQ_S] - jvs[638 * KQ_S] * x[12 * KQ_S] - jvs[639 * KQ_S] * x[13 * KQ_S] - jvs[640 * KQ_S] * x[119 * KQ_S] - jvs[641 * KQ_S] * x[120 * KQ_S] - jvs[642 * KQ_S] * x[121 * KQ_S] - jvs[643 * KQ_S] * x[126 * KQ_S] - jvs[644 * KQ_S] * x[127 * KQ_S] - jvs[645 * KQ_S] * x[142 * KQ_S] - jvs[646 * KQ_S] * x[143 * KQ_S] - jvs[647 * KQ_S] * x[144 * KQ_S] - jvs[648 * KQ_S] * x[145 * KQ_S] - jvs[649 * KQ_S] * x[147 * KQ_S] - jvs[650 * KQ_S] * x[148 * KQ_S] - jvs[651 * KQ_S] * x[149 * KQ_S] - jvs[652 * KQ_S] * x[150 * KQ_S] - jvs[653 * KQ_S] * x[152 * KQ_S] - jvs[654 * KQ_S] * x[153 * KQ_S] - jvs[655 * KQ_S] * x[154 * KQ_S] - jvs[656 * KQ_S] * x[155 * KQ_S];
    x[157 * KQ_S] = x[157 * KQ_S] - jvs[662 * KQ_S] * x[88 * KQ_S] - jvs[663 * KQ_S] * x[144 * KQ_S] - jvs[664 * KQ_S] * x[150 * KQ_S] - jvs[665 * KQ_S] * x[151 * KQ_S] - jvs[666 * KQ_S] * x[154 * KQ_S] - jvs[667 * KQ_S] * x[155 * KQ_S] - jvs[668 * KQ_S] * x[156 * KQ_S];
    x[158 * KQ_S] = x[158 * KQ_S] - jvs[673 * KQ_S] * x[95 * KQ_S] - jvs[674 * KQ_S] * x[125 * KQ_S] - jvs[675 * KQ_S] * x[144 * KQ_S] - jvs[676 * KQ_S] * x[146 * KQ_S] - jvs[677 * KQ_S] * x[149 * KQ_S] - jvs[678 * KQ_S] * x[150 * KQ_S] - jvs[679 * KQ_S] * x[151 * KQ_S] - jvs[680 * KQ_S] * x[153 * KQ_S] - jvs[681 * KQ_S] * x[154 * KQ_S] - jvs[682 * KQ_S] * x[155 * KQ_S] - jvs[683 * KQ_S] * x[156 * KQ_S] - jvs[684 * KQ_S] * x[157 * KQ_S];
    x[159 * KQ_S] = x[159 * KQ_S] - jvs[688 * KQ_S] * x[12 * KQ_S] - jvs[689 * KQ_S] * x[13 * KQ_S] - jvs[690 * KQ_S] * x[143 * KQ_S] - jvs[691 * KQ_S] * x[147 * KQ_S] - jvs[692 * KQ_S] * x[148 * KQ_S] - jvs[693 * KQ_S] * x[152 * KQ_S] - jvs[694 * KQ_S] * x[153 * KQ_S] - jvs[695 * KQ_S] * x[154 * KQ_S] - jvs[696 * KQ_S] * x[155 * KQ_S] - jvs[697 * KQ_S] * x[156 * KQ_S] - jvs[698 * KQ_S] * x[157 * KQ_S] - jvs[699 * KQ_S] * x[158 * KQ_S];
}

KQ_HD KQ_NOINLINE void kqu_solve_f2(const double* jvs, double* x)
{
    x[160 * KQ_S] = x[160 * KQ_S] - jvs[702 * KQ_S] * x[104 * KQ_S] - jvs[703 * KQ_S] * x[105 * KQ_S] - jvs[704 * KQ_S] * x[112 * KQ_S] - jvs[705 * KQ_S] * x[122 * KQ_S] - jvs[706 * KQ_S] * x[125 * KQ_S] - jvs[707 * KQ_S] * x[126 * KQ_S] - jvs[708 * KQ_S] * x[128 * KQ_S] - jvs[709 * KQ_S] * x[130 * KQ_S] - jvs[710 * KQ_S] * x[131 * KQ_S] - jvs[711 * KQ_S] * x[132 * KQ_S] - jvs[712 * KQ_S] * x[133 * KQ_S] - jvs[713 * KQ_S] * x[134 * KQ_S] - jvs[714 * KQ_S] * x[135 * KQ_S] - jvs[715 * KQ_S] * x[136 * KQ_S] - jvs[716 * KQ_S] * x[137 * KQ_S] - jvs[717 * KQ_S] * x[138 * KQ_S] - jvs[718 * KQ_S] * x[139 * KQ_S] - jvs[719 * KQ_S] * x[140 * KQ_S] - jvs[720 * KQ_S] * x[141 * KQ_S] - jvs[721 * KQ_S] * x[142 * KQ_S] - jvs[722 * KQ_S] * x[145 * KQ_S] - jvs[723 * KQ_S] * x[146 * KQ_S] - jvs[724 * KQ_S] * x[147 * KQ_S] - jvs[725 * KQ_S] * x[148 * KQ_S] - jvs[726 * KQ_S] * x[149 * KQ_S] - jvs[727 * KQ_S] * x[150 * KQ_S] - jvs[728 * KQ_S] * x[151 * KQ_S] - jvs[729 * KQ_S] * x[152 * KQ_S] - jvs[730 * KQ_S] * x[153 * KQ_S] - jvs[731 * KQ_S] * x[154 * KQ_S] - jvs[732 * KQ_S] * x[155 * KQ_S] - jvs[733 * KQ_S] * x[156 * KQ_S] - jvs[734 * KQ_S] * x[157 * KQ_S] - jvs[735 * KQ_S] * x[158 * KQ_S] - jvs[736 * KQ_S] * x[159 * KQ_S];
}

KQ_HD KQ_NOINLINE void kqu_solve_b0(const double* jvs, double* x)
{
    x[160 * KQ_S] = (x[160 * KQ_S]) / jvs[737 * KQ_S];
    x[159 * KQ_S] = (x[159 * KQ_S] - jvs[701 * KQ_S] * x[160 * KQ_S]) / jvs[700 * KQ_S];
    x[158 * KQ_S] = (x[158 * KQ_S] - jvs[686 * KQ_S] * x[159 * KQ_S] - jvs[687 * KQ_S] * x[160 * KQ_S]) / jvs[685 * KQ_S];
    x[157 * KQ_S] = (x[157 * KQ_S] - jvs[670 * KQ_S] * x[158 * KQ_S] - jvs[671 * KQ_S] * x[159 * KQ_S] - jvs[672 * KQ_S] * x[160 * KQ_S]) / jvs[669 * KQ_S];
    x[156 * KQ_S] = (x[156 * KQ_S] - jvs[658 * KQ_S] * x[157 * KQ_S] - jvs[659 * KQ_S] * x[158 * KQ_S] - jvs[660 * KQ_S] * x[159 * KQ_S] - jvs[661 * KQ_S] * x[160 * KQ_S]) / jvs[657 * KQ_S];
    x[155 * KQ_S] = (x[155 * KQ_S] - jvs[633 * KQ_S] * x[156 * KQ_S] - jvs[634 * KQ_S] * x[157 * KQ_S] - jvs[635 * KQ_S] * x[158 * KQ_S] - jvs[636 * KQ_S] * x[159 * KQ_S] - jvs[637 * KQ_S] * x[160 * KQ_S]) / jvs[632 * KQ_S];
    x[154 * KQ_S] = (x[154 * KQ_S] - jvs[585 * KQ_S] * x[155 * KQ_S] - jvs[586 * KQ_S] * x[156 * KQ_S] - jvs[587 * KQ_S] * x[157 * KQ_S] - jvs[588 * KQ_S] * x[158 * KQ_S] - jvs[589 * KQ_S] * x[159 * KQ_S] - jvs[590 * KQ_S] * x[160 * KQ_S]) / jvs[584 * KQ_S];
    x[153 * KQ_S] = (x[153 * KQ_S] - jvs[556 * KQ_S] * x[154 * KQ_S] - jvs[557 * KQ_S] * x[155 * KQ_S] - jvs[558 * KQ_S] * x[156 * KQ_S] - jvs[559 * KQ_S] * x[157 * KQ_S] - jvs[560 * KQ_S] * x[158 * KQ_S] - jvs[561 * KQ_S] * x[159 * KQ_S] - jvs[562 * KQ_S] * x[160 * KQ_S]) / jvs[555 * KQ_S];
    x[152 * KQ_S] = (x[152 * KQ_S] - jvs[529 * KQ_S] * x[153 * KQ_S] - jvs[530 * KQ_S] * x[154 * KQ_S] - jvs[531 * KQ_S] * x[155 * KQ_S] - jvs[532 * KQ_S] * x[156 * KQ_S] - jvs[533 * KQ_S] * x[157 * KQ_S] - jvs[534 * KQ_S] * x[158 * KQ_S] - jvs[535 * KQ_S] * x[159 * KQ_S] - jvs[536 * KQ_S] * x[160 * KQ_S]) / jvs[528 * KQ_S];
    x[151 * KQ_S] = (x[151 * KQ_S] - jvs[506 * KQ_S] * x[154 * KQ_S] - jvs[507 * KQ_S] * x[155 * KQ_S] - jvs[508 * KQ_S] * x[156 * KQ_S] - jvs[509 * KQ_S] * x[157 * KQ_S] - jvs[510 * KQ_S] * x[158 * KQ_S] - jvs[511 * KQ_S] * x[159 * KQ_S] - jvs[512 * KQ_S] * x[160 * KQ_S]) / jvs[505 * KQ_S];
    x[150 * KQ_S] = (x[150 * KQ_S] - jvs[495 * KQ_S] * x[154 * KQ_S] - jvs[496 * KQ_S] * x[155 * KQ_S] - jvs[497 * KQ_S] * x[157 * KQ_S] - jvs[498 * KQ_S] * x[158 * KQ_S] - jvs[499 * KQ_S] * x[160 * KQ_S]) / jvs[494 * KQ_S];
    x[149 * KQ_S] = (x[149 * KQ_S] - jvs[489 * KQ_S] * x[150 * KQ_S] - jvs[490 * KQ_S] * x[154 * KQ_S] - jvs[491 * KQ_S] * x[155 * KQ_S] - jvs[492 * KQ_S] * x[156 * KQ_S] - jvs[493 * KQ_S] * x[158 * KQ_S]) / jvs[488 * KQ_S];
    x[148 * KQ_S] = (x[148 * KQ_S] - jvs[481 * KQ_S] * x[152 * KQ_S] - jvs[482 * KQ_S] * x[155 * KQ_S] - jvs[483 * KQ_S] * x[156 * KQ_S] - jvs[484 * KQ_S] * x[159 * KQ_S] - jvs[485 * KQ_S] * x[160 * KQ_S]) / jvs[480 * KQ_S];
    x[147 * KQ_S] = (x[147 * KQ_S] - jvs[471 * KQ_S] * x[148 * KQ_S] - jvs[472 * KQ_S] * x[152 * KQ_S] - jvs[473 * KQ_S] * x[156 * KQ_S] - jvs[474 * KQ_S] * x[159 * KQ_S] - jvs[475 * KQ_S] * x[160 * KQ_S]) / jvs[470 * KQ_S];
    x[146 * KQ_S] = (x[146 * KQ_S] - jvs[463 * KQ_S] * x[149 * KQ_S] - jvs[464 * KQ_S] * x[151 * KQ_S] - jvs[465 * KQ_S] * x[153 * KQ_S] - jvs[466 * KQ_S] * x[155 * KQ_S] - jvs[467 * KQ_S] * x[156 * KQ_S] - jvs[468 * KQ_S] * x[157 * KQ_S]) / jvs[462 * KQ_S];
    x[145 * KQ_S] = (x[145 * KQ_S] - jvs[453 * KQ_S] * x[150 * KQ_S] - jvs[454 * KQ_S] * x[154 * KQ_S] - jvs[455 * KQ_S] * x[155 * KQ_S] - jvs[456 * KQ_S] * x[156 * KQ_S] - jvs[457 * KQ_S] * x[160 * KQ_S]) / jvs[452 * KQ_S];
    x[144 * KQ_S] = (x[144 * KQ_S] - jvs[447 * KQ_S] * x[155 * KQ_S] - jvs[448 * KQ_S] * x[156 * KQ_S] - jvs[449 * KQ_S] * x[157 * KQ_S] - jvs[450 * KQ_S] * x[158 * KQ_S]) / jvs[446 * KQ_S];
    x[143 * KQ_S] = (x[143 * KQ_S] - jvs[439 * KQ_S] * x[147 * KQ_S] - jvs[440 * KQ_S] * x[148 * KQ_S] - jvs[441 * KQ_S] * x[156 * KQ_S] - jvs[442 * KQ_S] * x[159 * KQ_S]) / jvs[438 * KQ_S];
    x[142 * KQ_S] = (x[142 * KQ_S] - jvs[432 * KQ_S] * x[153 * KQ_S] - jvs[433 * KQ_S] * x[154 * KQ_S] - jvs[434 * KQ_S] * x[156 * KQ_S] - jvs[435 * KQ_S] * x[160 * KQ_S]) / jvs[431 * KQ_S];
    x[141 * KQ_S] = (x[141 * KQ_S] - jvs[424 * KQ_S] * x[147 * KQ_S] - jvs[425 * KQ_S] * x[148 * KQ_S] - jvs[426 * KQ_S] * x[155 * KQ_S] - jvs[427 * KQ_S] * x[160 * KQ_S]) / jvs[423 * KQ_S];
    x[140 * KQ_S] = (x[140 * KQ_S] - jvs[419 * KQ_S] * x[155 * KQ_S] - jvs[420 * KQ_S] * x[160 * KQ_S]) / jvs[418 * KQ_S];
    x[139 * KQ_S] = (x[139 * KQ_S] - jvs[411 * KQ_S] * x[155 * KQ_S] - jvs[412 * KQ_S] * x[160 * KQ_S]) / jvs[410 * KQ_S];
    x[138 * KQ_S] = (x[138 * KQ_S] - jvs[406 * KQ_S] * x[139 * KQ_S] - jvs[407 * KQ_S] * x[155 * KQ_S] - jvs[408 * KQ_S] * x[160 * KQ_S]) / jvs[405 * KQ_S];
    x[137 * KQ_S] = (x[137 * KQ_S] - jvs[401 * KQ_S] * x[141 * KQ_S] - jvs[402 * KQ_S] * x[155 * KQ_S] - jvs[403 * KQ_S] * x[160 * KQ_S]) / jvs[400 * KQ_S];
    x[136 * KQ_S] = (x[136 * KQ_S] - jvs[397 * KQ_S] * x[140 * KQ_S] - jvs[398 * KQ_S] * x[155 * KQ_S] - jvs[399 * KQ_S] * x[160 * KQ_S]) / jvs[396 * KQ_S];
    x[135 * KQ_S] = (x[135 * KQ_S] - jvs[391 * KQ_S] * x[155 * KQ_S] - jvs[392 * KQ_S] * x[160 * KQ_S]) / jvs[390 * KQ_S];
    x[134 * KQ_S] = (x[134 * KQ_S] - jvs[384 * KQ_S] * x[135 * KQ_S] - jvs[385 * KQ_S] * x[155 * KQ_S] - jvs[386 * KQ_S] * x[160 * KQ_S]) / jvs[383 * KQ_S];
    x[133 * KQ_S] = (x[133 * KQ_S] - jvs[379 * KQ_S] * x[155 * KQ_S] - jvs[380 * KQ_S] * x[160 * KQ_S]) / jvs[378 * KQ_S];
    x[132 * KQ_S] = (x[132 * KQ_S] - jvs[373 * KQ_S] * x[133 * KQ_S] - jvs[374 * KQ_S] * x[155 * KQ_S] - jvs[375 * KQ_S] * x[160 * KQ_S]) / jvs[372 * KQ_S];
    x[131 * KQ_S] = (x[131 * KQ_S] - jvs[367 * KQ_S] * x[136 * KQ_S] - jvs[368 * KQ_S] * x[140 * KQ_S] - jvs[369 * KQ_S] * x[155 * KQ_S] - jvs[370 * KQ_S] * x[160 * KQ_S]) / jvs[366 * KQ_S];
    x[130 * KQ_S] = (x[130 * KQ_S] - jvs[361 * KQ_S] * x[131 * KQ_S] - jvs[362 * KQ_S] * x[155 * KQ_S] - jvs[363 * KQ_S] * x[160 * KQ_S]) / jvs[360 * KQ_S];
    x[129 * KQ_S] = (x[129 * KQ_S] - jvs[356 * KQ_S] * x[149 * KQ_S] - jvs[357 * KQ_S] * x[150 * KQ_S] - jvs[358 * KQ_S] * x[155 * KQ_S] - jvs[359 * KQ_S] * x[158 * KQ_S]) / jvs[355 * KQ_S];
    x[128 * KQ_S] = (x[128 * KQ_S] - jvs[351 * KQ_S] * x[131 * KQ_S] - jvs[352 * KQ_S] * x[136 * KQ_S] - jvs[353 * KQ_S] * x[155 * KQ_S] - jvs[354 * KQ_S] * x[160 * KQ_S]) / jvs[350 * KQ_S];
    x[127 * KQ_S] = (x[127 * KQ_S] - jvs[346 * KQ_S] * x[142 * KQ_S] - jvs[347 * KQ_S] * x[154 * KQ_S] - jvs[348 * KQ_S] * x[155 * KQ_S] - jvs[349 * KQ_S] * x[156 * KQ_S]) / jvs[345 * KQ_S];
    x[126 * KQ_S] = (x[126 * KQ_S] - jvs[343 * KQ_S] * x[153 * KQ_S] - jvs[344 * KQ_S] * x[156 * KQ_S]) / jvs[342 * KQ_S];
    x[125 * KQ_S] = (x[125 * KQ_S] - jvs[338 * KQ_S] * x[151 * KQ_S] - jvs[339 * KQ_S] * x[155 * KQ_S] - jvs[340 * KQ_S] * x[160 * KQ_S]) / jvs[337 * KQ_S];
    x[124 * KQ_S] = (x[124 * KQ_S] - jvs[327 * KQ_S] * x[128 * KQ_S] - jvs[328 * KQ_S] * x[130 * KQ_S] - jvs[329 * KQ_S] * x[131 * KQ_S] - jvs[330 * KQ_S] * x[132 * KQ_S] - jvs[331 * KQ_S] * x[133 * KQ_S] - jvs[332 * KQ_S] * x[137 * KQ_S] - jvs[333 * KQ_S] * x[141 * KQ_S] - jvs[334 * KQ_S] * x[155 * KQ_S] - jvs[335 * KQ_S] * x[160 * KQ_S]) / jvs[326 * KQ_S];
    x[123 * KQ_S] = (x[123 * KQ_S] - jvs[320 * KQ_S] * x[126 * KQ_S] - jvs[321 * KQ_S] * x[142 * KQ_S] - jvs[322 * KQ_S] * x[153 * KQ_S] - jvs[323 * KQ_S] * x[155 * KQ_S]) / jvs[319 * KQ_S];
    x[122 * KQ_S] = (x[122 * KQ_S] - jvs[314 * KQ_S] * x[126 * KQ_S] - jvs[315 * KQ_S] * x[142 * KQ_S] - jvs[316 * KQ_S] * x[153 * KQ_S]) / jvs[313 * KQ_S];
    x[121 * KQ_S] = (x[121 * KQ_S] - jvs[311 * KQ_S] * x[155 * KQ_S] - jvs[312 * KQ_S] * x[156 * KQ_S]) / jvs[310 * KQ_S];
    x[120 * KQ_S] = (x[120 * KQ_S] - jvs[307 * KQ_S] * x[155 * KQ_S] - jvs[308 * KQ_S] * x[156 * KQ_S]) / jvs[306 * KQ_S];
    x[119 * KQ_S] = (x[119 * KQ_S] - jvs[303 * KQ_S] * x[156 * KQ_S]) / jvs[302 * KQ_S];
}

KQ_HD KQ_NOINLINE void kqu_solve_b1(const double* jvs, double* x)
{
    x[118 * KQ_S] = (x[118 * KQ_S] - jvs[297 * KQ_S] * x[152 * KQ_S] - jvs[298 * KQ_S] * x[156 * KQ_S] - jvs[299 * KQ_S] * x[159 * KQ_S] - jvs[300 * KQ_S] * x[160 * KQ_S]) / jvs[296 * KQ_S];
    x[117 * KQ_S] = (x[117 * KQ_S] - jvs[288 * KQ_S] * x[118 * KQ_S] - jvs[289 * KQ_S] * x[152 * KQ_S] - jvs[290 * KQ_S] * x[156 * KQ_S] - jvs[291 * KQ_S] * x[159 * KQ_S] - jvs[292 * KQ_S] * x[160 * KQ_S]) / jvs[287 * KQ_S];
    x[116 * KQ_S] = (x[116 * KQ_S] - jvs[283 * KQ_S] * x[117 * KQ_S] - jvs[284 * KQ_S] * x[118 * KQ_S] - jvs[285 * KQ_S] * x[152 * KQ_S] - jvs[286 * KQ_S] * x[160 * KQ_S]) / jvs[282 * KQ_S];
    x[115 * KQ_S] = (x[115 * KQ_S] - jvs[280 * KQ_S] * x[146 * KQ_S] - jvs[281 * KQ_S] * x[153 * KQ_S]) / jvs[279 * KQ_S];
    x[114 * KQ_S] = (x[114 * KQ_S] - jvs[274 * KQ_S] * x[124 * KQ_S] - jvs[275 * KQ_S] * x[155 * KQ_S]) / jvs[273 * KQ_S];
    x[113 * KQ_S] = (x[113 * KQ_S] - jvs[270 * KQ_S] * x[114 * KQ_S] - jvs[271 * KQ_S] * x[155 * KQ_S]) / jvs[269 * KQ_S];
    x[112 * KQ_S] = (x[112 * KQ_S] - jvs[268 * KQ_S] * x[160 * KQ_S]) / jvs[267 * KQ_S];
    x[111 * KQ_S] = (x[111 * KQ_S] - jvs[265 * KQ_S] * x[155 * KQ_S]) / jvs[264 * KQ_S];
    x[110 * KQ_S] = (x[110 * KQ_S] - jvs[260 * KQ_S] * x[111 * KQ_S] - jvs[261 * KQ_S] * x[155 * KQ_S]) / jvs[259 * KQ_S];
    x[109 * KQ_S] = (x[109 * KQ_S] - jvs[256 * KQ_S] * x[123 * KQ_S] - jvs[257 * KQ_S] * x[155 * KQ_S]) / jvs[255 * KQ_S];
    x[108 * KQ_S] = (x[108 * KQ_S] - jvs[254 * KQ_S] * x[152 * KQ_S]) / jvs[253 * KQ_S];
    x[107 * KQ_S] = (x[107 * KQ_S] - jvs[249 * KQ_S] * x[108 * KQ_S] - jvs[250 * KQ_S] * x[152 * KQ_S]) / jvs[248 * KQ_S];
    x[106 * KQ_S] = (x[106 * KQ_S] - jvs[245 * KQ_S] * x[146 * KQ_S] - jvs[246 * KQ_S] * x[155 * KQ_S]) / jvs[244 * KQ_S];
    x[105 * KQ_S] = (x[105 * KQ_S] - jvs[242 * KQ_S] * x[160 * KQ_S]) / jvs[241 * KQ_S];
    x[104 * KQ_S] = (x[104 * KQ_S] - jvs[238 * KQ_S] * x[160 * KQ_S]) / jvs[237 * KQ_S];
    x[103 * KQ_S] = (x[103 * KQ_S] - jvs[232 * KQ_S] * x[119 * KQ_S] - jvs[233 * KQ_S] * x[126 * KQ_S] - jvs[234 * KQ_S] * x[156 * KQ_S] - jvs[235 * KQ_S] * x[160 * KQ_S]) / jvs[231 * KQ_S];
    x[102 * KQ_S] = (x[102 * KQ_S] - jvs[229 * KQ_S] * x[115 * KQ_S] - jvs[230 * KQ_S] * x[153 * KQ_S]) / jvs[228 * KQ_S];
    x[101 * KQ_S] = (x[101 * KQ_S] - jvs[227 * KQ_S] * x[115 * KQ_S]) / jvs[226 * KQ_S];
    x[100 * KQ_S] = (x[100 * KQ_S] - jvs[225 * KQ_S] * x[115 * KQ_S]) / jvs[224 * KQ_S];
    x[99 * KQ_S] = (x[99 * KQ_S] - jvs[223 * KQ_S] * x[144 * KQ_S]) / jvs[222 * KQ_S];
    x[98 * KQ_S] = (x[98 * KQ_S] - jvs[221 * KQ_S] * x[119 * KQ_S]) / jvs[220 * KQ_S];
    x[97 * KQ_S] = (x[97 * KQ_S] - jvs[219 * KQ_S] * x[126 * KQ_S]) / jvs[218 * KQ_S];
    x[96 * KQ_S] = (x[96 * KQ_S] - jvs[217 * KQ_S] * x[149 * KQ_S]) / jvs[216 * KQ_S];
    x[95 * KQ_S] = (x[95 * KQ_S] - jvs[215 * KQ_S] * x[158 * KQ_S]) / jvs[214 * KQ_S];
    x[94 * KQ_S] = (x[94 * KQ_S] - jvs[213 * KQ_S] * x[112 * KQ_S]) / jvs[212 * KQ_S];
    x[93 * KQ_S] = (x[93 * KQ_S] - jvs[211 * KQ_S] * x[105 * KQ_S]) / jvs[210 * KQ_S];
    x[92 * KQ_S] = (x[92 * KQ_S] - jvs[209 * KQ_S] * x[110 * KQ_S]) / jvs[208 * KQ_S];
    x[91 * KQ_S] = (x[91 * KQ_S] - jvs[207 * KQ_S] * x[121 * KQ_S]) / jvs[206 * KQ_S];
    x[90 * KQ_S] = (x[90 * KQ_S] - jvs[205 * KQ_S] * x[120 * KQ_S]) / jvs[204 * KQ_S];
    x[89 * KQ_S] = (x[89 * KQ_S] - jvs[203 * KQ_S] * x[141 * KQ_S]) / jvs[202 * KQ_S];
    x[88 * KQ_S] = (x[88 * KQ_S] - jvs[201 * KQ_S] * x[157 * KQ_S]) / jvs[200 * KQ_S];
    x[87 * KQ_S] = (x[87 * KQ_S] - jvs[199 * KQ_S] * x[107 * KQ_S]) / jvs[198 * KQ_S];
    x[86 * KQ_S] = (x[86 * KQ_S] - jvs[197 * KQ_S] * x[124 * KQ_S]) / jvs[196 * KQ_S];
    x[85 * KQ_S] = (x[85 * KQ_S] - jvs[195 * KQ_S] * x[106 * KQ_S]) / jvs[194 * KQ_S];
    x[84 * KQ_S] = (x[84 * KQ_S] - jvs[193 * KQ_S] * x[145 * KQ_S]) / jvs[192 * KQ_S];
    x[83 * KQ_S] = (x[83 * KQ_S] - jvs[191 * KQ_S] * x[118 * KQ_S]) / jvs[190 * KQ_S];
    x[82 * KQ_S] = (x[82 * KQ_S] - jvs[189 * KQ_S] * x[133 * KQ_S]) / jvs[188 * KQ_S];
    x[81 * KQ_S] = (x[81 * KQ_S] - jvs[187 * KQ_S] * x[154 * KQ_S]) / jvs[186 * KQ_S];
    x[80 * KQ_S] = (x[80 * KQ_S] - jvs[185 * KQ_S] * x[143 * KQ_S]) / jvs[184 * KQ_S];
    x[79 * KQ_S] = (x[79 * KQ_S] - jvs[183 * KQ_S] * x[134 * KQ_S]) / jvs[182 * KQ_S];
    x[78 * KQ_S] = (x[78 * KQ_S] - jvs[181 * KQ_S] * x[104 * KQ_S]) / jvs[180 * KQ_S];
    x[77 * KQ_S] = (x[77 * KQ_S] - jvs[179 * KQ_S] * x[153 * KQ_S]) / jvs[178 * KQ_S];
    x[76 * KQ_S] = (x[76 * KQ_S] - jvs[176 * KQ_S] * x[77 * KQ_S]) / jvs[175 * KQ_S];
    x[75 * KQ_S] = (x[75 * KQ_S] - jvs[174 * KQ_S] * x[153 * KQ_S]) / jvs[173 * KQ_S];
    x[74 * KQ_S] = (x[74 * KQ_S] - jvs[171 * KQ_S] * x[75 * KQ_S]) / jvs[170 * KQ_S];
    x[73 * KQ_S] = (x[73 * KQ_S] - jvs[169 * KQ_S] * x[125 * KQ_S]) / jvs[168 * KQ_S];
    x[72 * KQ_S] = (x[72 * KQ_S] - jvs[167 * KQ_S] * x[119 * KQ_S]) / jvs[166 * KQ_S];
    x[71 * KQ_S] = (x[71 * KQ_S] - jvs[165 * KQ_S] * x[126 * KQ_S]) / jvs[164 * KQ_S];
    x[70 * KQ_S] = (x[70 * KQ_S] - jvs[161 * KQ_S] * x[116 * KQ_S] - jvs[162 * KQ_S] * x[117 * KQ_S] - jvs[163 * KQ_S] * x[118 * KQ_S]) / jvs[160 * KQ_S];
    x[69 * KQ_S] = (x[69 * KQ_S] - jvs[158 * KQ_S] * x[138 * KQ_S] - jvs[159 * KQ_S] * x[139 * KQ_S]) / jvs[157 * KQ_S];
    x[68 * KQ_S] = (x[68 * KQ_S] - jvs[156 * KQ_S] * x[104 * KQ_S]) / jvs[155 * KQ_S];
    x[67 * KQ_S] = (x[67 * KQ_S] - jvs[153 * KQ_S] * x[150 * KQ_S] - jvs[154 * KQ_S] * x[154 * KQ_S]) / jvs[152 * KQ_S];
    x[66 * KQ_S] = (x[66 * KQ_S] - jvs[149 * KQ_S] * x[143 * KQ_S] - jvs[150 * KQ_S] * x[147 * KQ_S] - jvs[151 * KQ_S] * x[148 * KQ_S]) / jvs[148 * KQ_S];
    x[65 * KQ_S] = (x[65 * KQ_S] - jvs[146 * KQ_S] * x[134 * KQ_S] - jvs[147 * KQ_S] * x[135 * KQ_S]) / jvs[145 * KQ_S];
    x[64 * KQ_S] = (x[64 * KQ_S] - jvs[143 * KQ_S] * x[132 * KQ_S] - jvs[144 * KQ_S] * x[133 * KQ_S]) / jvs[142 * KQ_S];
    x[63 * KQ_S] = (x[63 * KQ_S] - jvs[139 * KQ_S] * x[128 * KQ_S] - jvs[140 * KQ_S] * x[130 * KQ_S] - jvs[141 * KQ_S] * x[131 * KQ_S]) / jvs[138 * KQ_S];
    x[62 * KQ_S] = (x[62 * KQ_S] - jvs[136 * KQ_S] * x[136 * KQ_S] - jvs[137 * KQ_S] * x[140 * KQ_S]) / jvs[135 * KQ_S];
    x[61 * KQ_S] = (x[61 * KQ_S] - jvs[132 * KQ_S] * x[75 * KQ_S] - jvs[133 * KQ_S] * x[77 * KQ_S] - jvs[134 * KQ_S] * x[153 * KQ_S]) / jvs[131 * KQ_S];
    x[60 * KQ_S] = (x[60 * KQ_S] - jvs[130 * KQ_S] * x[61 * KQ_S]) / jvs[129 * KQ_S];
    x[59 * KQ_S] = (x[59 * KQ_S] - jvs[127 * KQ_S] * x[75 * KQ_S] - jvs[128 * KQ_S] * x[77 * KQ_S]) / jvs[126 * KQ_S];
    x[58 * KQ_S] = (x[58 * KQ_S] - jvs[125 * KQ_S] * x[59 * KQ_S]) / jvs[124 * KQ_S];
    x[57 * KQ_S] = (x[57 * KQ_S] - jvs[123 * KQ_S] * x[77 * KQ_S]) / jvs[122 * KQ_S];
    x[56 * KQ_S] = (x[56 * KQ_S] - jvs[121 * KQ_S] * x[75 * KQ_S]) / jvs[120 * KQ_S];
    x[55 * KQ_S] = (x[55 * KQ_S] - jvs[117 * KQ_S] * x[101 * KQ_S] - jvs[118 * KQ_S] * x[102 * KQ_S] - jvs[119 * KQ_S] * x[115 * KQ_S]) / jvs[116 * KQ_S];
    x[54 * KQ_S] = (x[54 * KQ_S] - jvs[115 * KQ_S] * x[55 * KQ_S]) / jvs[114 * KQ_S];
    x[53 * KQ_S] = (x[53 * KQ_S] - jvs[113 * KQ_S] * x[102 * KQ_S]) / jvs[112 * KQ_S];
    x[52 * KQ_S] = (x[52 * KQ_S] - jvs[109 * KQ_S] * x[115 * KQ_S] - jvs[110 * KQ_S] * x[146 * KQ_S] - jvs[111 * KQ_S] * x[153 * KQ_S]) / jvs[108 * KQ_S];
    x[51 * KQ_S] = (x[51 * KQ_S] - jvs[106 * KQ_S] * x[52 * KQ_S] - jvs[107 * KQ_S] * x[101 * KQ_S]) / jvs[105 * KQ_S];
    x[50 * KQ_S] = (x[50 * KQ_S] - jvs[104 * KQ_S] * x[115 * KQ_S]) / jvs[103 * KQ_S];
    x[49 * KQ_S] = (x[49 * KQ_S] - jvs[101 * KQ_S] * x[129 * KQ_S] - jvs[102 * KQ_S] * x[149 * KQ_S]) / jvs[100 * KQ_S];
    x[48 * KQ_S] = (x[48 * KQ_S] - jvs[98 * KQ_S] * x[125 * KQ_S] - jvs[99 * KQ_S] * x[151 * KQ_S]) / jvs[97 * KQ_S];
    x[47 * KQ_S] = (x[47 * KQ_S] - jvs[96 * KQ_S] * x[158 * KQ_S]) / jvs[95 * KQ_S];
    x[46 * KQ_S] = (x[46 * KQ_S]) / jvs[94 * KQ_S];
    x[45 * KQ_S] = (x[45 * KQ_S]) / jvs[92 * KQ_S];
    x[44 * KQ_S] = (x[44 * KQ_S]) / jvs[90 * KQ_S];
    x[43 * KQ_S] = (x[43 * KQ_S]) / jvs[88 * KQ_S];
    x[42 * KQ_S] = (x[42 * KQ_S] - jvs[86 * KQ_S] * x[155 * KQ_S]) / jvs[85 * KQ_S];
    x[41 * KQ_S] = (x[41 * KQ_S]) / jvs[84 * KQ_S];
    x[40 * KQ_S] = (x[40 * KQ_S]) / jvs[82 * KQ_S];
    x[39 * KQ_S] = (x[39 * KQ_S]) / jvs[80 * KQ_S];
    x[38 * KQ_S] = (x[38 * KQ_S]) / jvs[78 * KQ_S];
    x[37 * KQ_S] = (x[37 * KQ_S]) / jvs[76 * KQ_S];
    x[36 * KQ_S] = (x[36 * KQ_S]) / jvs[74 * KQ_S];
    x[35 * KQ_S] = (x[35 * KQ_S] - jvs[72 * KQ_S] * x[111 * KQ_S]) / jvs[71 * KQ_S];
}

KQ_HD KQ_NOINLINE void kqu_solve_b2(const double* jvs, double* x)
{
    x[34 * KQ_S] = (x[34 * KQ_S] - jvs[70 * KQ_S] * x[108 * KQ_S]) / jvs[69 * KQ_S];
    x[33 * KQ_S] = (x[33 * KQ_S] - jvs[68 * KQ_S] * x[146 * KQ_S]) / jvs[67 * KQ_S];
    x[32 * KQ_S] = (x[32 * KQ_S] - jvs[66 * KQ_S] * x[160 * KQ_S]) / jvs[65 * KQ_S];
    x[31 * KQ_S] = (x[31 * KQ_S] - jvs[64 * KQ_S] * x[112 * KQ_S]) / jvs[63 * KQ_S];
    x[30 * KQ_S] = (x[30 * KQ_S] - jvs[62 * KQ_S] * x[105 * KQ_S]) / jvs[61 * KQ_S];
    x[29 * KQ_S] = (x[29 * KQ_S] - jvs[60 * KQ_S] * x[110 * KQ_S]) / jvs[59 * KQ_S];
    x[28 * KQ_S] = (x[28 * KQ_S] - jvs[56 * KQ_S] * x[109 * KQ_S] - jvs[57 * KQ_S] * x[123 * KQ_S] - jvs[58 * KQ_S] * x[153 * KQ_S]) / jvs[55 * KQ_S];
    x[27 * KQ_S] = (x[27 * KQ_S] - jvs[54 * KQ_S] * x[121 * KQ_S]) / jvs[53 * KQ_S];
    x[26 * KQ_S] = (x[26 * KQ_S] - jvs[52 * KQ_S] * x[120 * KQ_S]) / jvs[51 * KQ_S];
    x[25 * KQ_S] = (x[25 * KQ_S] - jvs[49 * KQ_S] * x[137 * KQ_S] - jvs[50 * KQ_S] * x[141 * KQ_S]) / jvs[48 * KQ_S];
    x[24 * KQ_S] = (x[24 * KQ_S] - jvs[47 * KQ_S] * x[157 * KQ_S]) / jvs[46 * KQ_S];
    x[23 * KQ_S] = (x[23 * KQ_S] - jvs[45 * KQ_S] * x[145 * KQ_S]) / jvs[44 * KQ_S];
    x[22 * KQ_S] = (x[22 * KQ_S] - jvs[43 * KQ_S] * x[107 * KQ_S]) / jvs[42 * KQ_S];
    x[21 * KQ_S] = (x[21 * KQ_S] - jvs[39 * KQ_S] * x[130 * KQ_S] - jvs[40 * KQ_S] * x[131 * KQ_S] - jvs[41 * KQ_S] * x[160 * KQ_S]) / jvs[38 * KQ_S];
    x[20 * KQ_S] = (x[20 * KQ_S] - jvs[34 * KQ_S] * x[21 * KQ_S] - jvs[35 * KQ_S] * x[113 * KQ_S] - jvs[36 * KQ_S] * x[114 * KQ_S] - jvs[37 * KQ_S] * x[124 * KQ_S]) / jvs[33 * KQ_S];
    x[19 * KQ_S] = (x[19 * KQ_S] - jvs[32 * KQ_S] * x[106 * KQ_S]) / jvs[31 * KQ_S];
    x[18 * KQ_S] = (x[18 * KQ_S] - jvs[23 * KQ_S] * x[103 * KQ_S] - jvs[24 * KQ_S] * x[122 * KQ_S] - jvs[25 * KQ_S] * x[127 * KQ_S] - jvs[26 * KQ_S] * x[142 * KQ_S] - jvs[27 * KQ_S] * x[144 * KQ_S] - jvs[28 * KQ_S] * x[147 * KQ_S] - jvs[29 * KQ_S] * x[156 * KQ_S] - jvs[30 * KQ_S] * x[159 * KQ_S]) / jvs[22 * KQ_S];
    x[17 * KQ_S] = (x[17 * KQ_S]) / jvs[21 * KQ_S];
    x[16 * KQ_S] = (x[16 * KQ_S]) / jvs[19 * KQ_S];
    x[15 * KQ_S] = (x[15 * KQ_S]) / jvs[18 * KQ_S];
    x[14 * KQ_S] = (x[14 * KQ_S]) / jvs[17 * KQ_S];
    x[13 * KQ_S] = (x[13 * KQ_S]) / jvs[16 * KQ_S];
    x[12 * KQ_S] = (x[12 * KQ_S]) / jvs[15 * KQ_S];
    x[11 * KQ_S] = (x[11 * KQ_S]) / jvs[14 * KQ_S];
    x[10 * KQ_S] = (x[10 * KQ_S]) / jvs[12 * KQ_S];
    x[9 * KQ_S] = (x[9 * KQ_S]) / jvs[11 * KQ_S];
    x[8 * KQ_S] = (x[8 * KQ_S]) / jvs[9 * KQ_S];
    x[7 * KQ_S] = (x[7 * KQ_S]) / jvs[7 * KQ_S];
    x[6 * KQ_S] = (x[6 * KQ_S]) / jvs[6 * KQ_S];
    x[5 * KQ_S] = (x[5 * KQ_S]) / jvs[5 * KQ_S];
    x[4 * KQ_S] = (x[4 * KQ_S]) / jvs[4 * KQ_S];
    x[3 * KQ_S] = (x[3 * KQ_S]) / jvs[3 * KQ_S];
    x[2 * KQ_S] = (x[2 * KQ_S]) / jvs[2 * KQ_S];
    x[1 * KQ_S] = (x[1 * KQ_S]) / jvs[1 * KQ_S];
    x[0 * KQ_S] = (x[0 * KQ_S]) / jvs[0 * KQ_S];
}

KQ_HD inline void kqu_solve(const double* jvs, double* x)
{
    kqu_solve_f0(jvs, x);
    kqu_solve_f1(jvs, x);
    kqu_solve_f2(jvs, x);
    kqu_solve_b0(jvs, x);
    kqu_solve_b1(jvs, x);
    kqu_solve_b2(jvs, x);
}
