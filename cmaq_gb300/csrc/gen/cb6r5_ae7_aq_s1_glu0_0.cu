// Generated by cmaq_gb300.mechgen.generate from CCTM/src/MECHS/cb6r5_ae7_aq/RXNS_DATA_MODULE.F90
// and RXNS_FUNC_MODULE.F90 (sha256/16 4242f44b2527a299).  Do not edit.
#include "cb6r5_ae7_aq_mech.cuh"
#include <math.h>
namespace mech_cb6r5_ae7_aq {
__device__ __noinline__ void gear_pdecomp_s1_0_0(double* __restrict__ ws, double r1delt)
{
    double* __restrict__ lu = ws + 2426;
    double* __restrict__ vd = ws + 4116;
    { // row 0
      double a0 = 1.0;
      a0 = fma(-r1delt, ws[1334], a0);
      vd[0] = 1.0 / a0;
    }
    { // row 1
      double a0 = 0.0;
      a0 = fma(r1delt, ws[1334], a0);
      double a1 = 1.0;
      a0 = a0 * CHEM_LDLU(vd + 0);
      lu[1] = a0;
      vd[1] = 1.0 / a1;
    }
    { // row 2
      double a2 = 1.0;
      a2 = fma(-r1delt, ws[1335], a2);
      vd[2] = 1.0 / a2;
    }
    { // row 3
      double a3 = 1.0;
      a3 = fma(-r1delt, ws[1336], a3);
      vd[3] = 1.0 / a3;
    }
    { // row 4
      double a4 = 1.0;
      a4 = fma(-r1delt, ws[1337], a4);
      vd[4] = 1.0 / a4;
    }
    { // row 5
      double a5 = 1.0;
      a5 = fma(-r1delt, ws[1338], a5);
      vd[5] = 1.0 / a5;
    }
    { // row 6
      double a6 = 1.0;
      a6 = fma(-r1delt, ws[1339], a6);
      vd[6] = 1.0 / a6;
    }
    { // row 7
      double a7 = 1.0;
      a7 = fma(-r1delt, ws[1340], a7);
      vd[7] = 1.0 / a7;
    }
    { // row 8
      double a8 = 1.0;
      double a69 = 0.0;
      a69 = fma(r1delt, ws[1811], a69);
      double a148 = 0.0;
      a148 = fma(r1delt, ws[1812], a148);
      lu[1539] = a69;
      lu[1540] = a148;
      vd[8] = 1.0 / a8;
    }
    { // row 9
      double a9 = 1.0;
      double a69 = 0.0;
      a69 = fma(r1delt, ws[1811], a69);
      double a148 = 0.0;
      a148 = fma(r1delt, ws[1812], a148);
      lu[1537] = a69;
      lu[1538] = a148;
      vd[9] = 1.0 / a9;
    }
    { // row 10
      double a10 = 1.0;
      a10 = fma(-r1delt, ws[1170], a10);
      double a30 = 0.0;
      a30 = fma(0.2 * r1delt, ws[1175], a30);
      a30 = fma(r1delt, ws[1176], a30);
      lu[1536] = a30;
      vd[10] = 1.0 / a10;
    }
    { // row 11
      double a11 = 1.0;
      a11 = fma(-r1delt, ws[1937], a11);
      double a148 = 0.0;
      a148 = fma(-r1delt, ws[1938], a148);
      lu[1535] = a148;
      vd[11] = 1.0 / a11;
    }
    { // row 12
      double a12 = 1.0;
      a12 = fma(-r1delt, ws[2017], a12);
      double a148 = 0.0;
      a148 = fma(-r1delt, ws[2018], a148);
      lu[1534] = a148;
      vd[12] = 1.0 / a12;
    }
    { // row 13
      double a13 = 1.0;
      a13 = fma(-r1delt, ws[2091], a13);
      double a148 = 0.0;
      a148 = fma(-r1delt, ws[2092], a148);
      lu[1533] = a148;
      vd[13] = 1.0 / a13;
    }
    { // row 14
      double a14 = 1.0;
      a14 = fma(-r1delt, ws[2163], a14);
      double a148 = 0.0;
      a148 = fma(-r1delt, ws[2164], a148);
      lu[1532] = a148;
      vd[14] = 1.0 / a14;
    }
    { // row 15
      double a15 = 1.0;
      a15 = fma(-r1delt, ws[2166], a15);
      double a60 = 0.0;
      a60 = fma(-r1delt, ws[2165], a60);
      lu[1531] = a60;
      vd[15] = 1.0 / a15;
    }
    { // row 16
      double a16 = 1.0;
      a16 = fma(-r1delt, ws[2168], a16);
      double a60 = 0.0;
      a60 = fma(-r1delt, ws[2167], a60);
      lu[1530] = a60;
      vd[16] = 1.0 / a16;
    }
    { // row 17
      double a17 = 1.0;
      a17 = fma(-r1delt, ws[2170], a17);
      double a39 = 0.0;
      a39 = fma(-r1delt, ws[2169], a39);
      lu[1529] = a39;
      vd[17] = 1.0 / a17;
    }
    { // row 18
      double a18 = 1.0;
      a18 = fma(-r1delt, ws[2172], a18);
      double a41 = 0.0;
      a41 = fma(-r1delt, ws[2171], a41);
      lu[1528] = a41;
      vd[18] = 1.0 / a18;
    }
    { // row 19
      double a18 = 0.0;
      a18 = fma(r1delt, ws[2172], a18);
      double a19 = 1.0;
      double a41 = 0.0;
      a41 = fma(r1delt, ws[2171], a41);
      a41 = fma(r1delt, ws[1324], a41);
      a18 = a18 * CHEM_LDLU(vd + 18);
      lu[2] = a18;
      a41 = fma(-a18, CHEM_LDLU(lu + 1528), a41);
      lu[1527] = a41;
      vd[19] = 1.0 / a19;
    }
    { // row 20
      double a20 = 1.0;
      double a125 = 0.0;
      a125 = fma(r1delt, ws[1326], a125);
      double a133 = 0.0;
      a133 = fma(r1delt, ws[1325], a133);
      lu[1525] = a125;
      lu[1526] = a133;
      vd[20] = 1.0 / a20;
    }
    { // row 21
      double a21 = 1.0;
      a21 = fma(-r1delt, ws[1052], a21);
      a21 = fma(-r1delt, ws[1053], a21);
      double a135 = 0.0;
      a135 = fma(r1delt, ws[1051], a135);
      lu[1524] = a135;
      vd[21] = 1.0 / a21;
    }
    { // row 22
      double a22 = 1.0;
      a22 = fma(-r1delt, ws[2185], a22);
      a22 = fma(r1delt, ws[2185], a22);
      double a148 = 0.0;
      a148 = fma(-r1delt, ws[2186], a148);
      a148 = fma(r1delt, ws[2186], a148);
      lu[1523] = a148;
      vd[22] = 1.0 / a22;
    }
    { // row 23
      double a23 = 1.0;
      a23 = fma(-r1delt, ws[2189], a23);
      a23 = fma(r1delt, ws[2189], a23);
      double a148 = 0.0;
      a148 = fma(-r1delt, ws[2190], a148);
      a148 = fma(r1delt, ws[2190], a148);
      lu[1522] = a148;
      vd[23] = 1.0 / a23;
    }
    { // row 24
      double a24 = 1.0;
      a24 = fma(-r1delt, ws[2193], a24);
      double a148 = 0.0;
      a148 = fma(-r1delt, ws[2194], a148);
      lu[1521] = a148;
      vd[24] = 1.0 / a24;
    }
    { // row 25
      double a24 = 0.0;
      a24 = fma(r1delt, ws[2193], a24);
      double a25 = 1.0;
      double a148 = 0.0;
      a148 = fma(r1delt, ws[2194], a148);
      a24 = a24 * CHEM_LDLU(vd + 24);
      lu[3] = a24;
      a148 = fma(-a24, CHEM_LDLU(lu + 1521), a148);
      lu[1520] = a148;
      vd[25] = 1.0 / a25;
    }
    { // row 26
      double a26 = 1.0;
      a26 = fma(-r1delt, ws[1923], a26);
      a26 = fma(-r1delt, ws[2112], a26);
      double a142 = 0.0;
      a142 = fma(-r1delt, ws[2111], a142);
      double a148 = 0.0;
      a148 = fma(-r1delt, ws[1924], a148);
      lu[1518] = a142;
      lu[1519] = a148;
      vd[26] = 1.0 / a26;
    }
    { // row 27
      double a27 = 1.0;
      a27 = fma(-r1delt, ws[1927], a27);
      a27 = fma(-r1delt, ws[2130], a27);
      double a142 = 0.0;
      a142 = fma(-r1delt, ws[2129], a142);
      double a148 = 0.0;
      a148 = fma(-r1delt, ws[1928], a148);
      lu[1516] = a142;
      lu[1517] = a148;
      vd[27] = 1.0 / a27;
    }
    { // row 28
      double a28 = 1.0;
      a28 = fma(-r1delt, ws[1931], a28);
      a28 = fma(-r1delt, ws[2110], a28);
      double a142 = 0.0;
      a142 = fma(-r1delt, ws[2109], a142);
      double a148 = 0.0;
      a148 = fma(-r1delt, ws[1932], a148);
      lu[1514] = a142;
      lu[1515] = a148;
      vd[28] = 1.0 / a28;
    }
    { // row 29
      double a28 = 0.0;
      a28 = fma(r1delt, ws[1931], a28);
      double a29 = 1.0;
      a29 = fma(-r1delt, ws[1263], a29);
      a29 = fma(-r1delt, ws[1264], a29);
      double a142 = 0.0;
      double a148 = 0.0;
      a148 = fma(r1delt, ws[1932], a148);
      a28 = a28 * CHEM_LDLU(vd + 28);
      lu[4] = a28;
      a142 = fma(-a28, CHEM_LDLU(lu + 1514), a142);
      a148 = fma(-a28, CHEM_LDLU(lu + 1515), a148);
      lu[1512] = a142;
      lu[1513] = a148;
      vd[29] = 1.0 / a29;
    }
    { // row 30
      double a30 = 1.0;
      a30 = fma(-r1delt, ws[1175], a30);
      a30 = fma(0.02 * r1delt, ws[1175], a30);
      a30 = fma(-r1delt, ws[1176], a30);
      a30 = fma(-r1delt, ws[1935], a30);
      double a62 = 0.0;
      a62 = fma(0.874 * r1delt, ws[1266], a62);
      double a144 = 0.0;
      a144 = fma(-r1delt, ws[1936], a144);
      lu[1510] = a62;
      lu[1511] = a144;
      vd[30] = 1.0 / a30;
    }
    { // row 31
      double a31 = 1.0;
      double a79 = 0.0;
      a79 = fma(r1delt, ws[1963], a79);
      a79 = fma(r1delt, ws[1977], a79);
      double a145 = 0.0;
      a145 = fma(r1delt, ws[1978], a145);
      double a148 = 0.0;
      a148 = fma(r1delt, ws[1964], a148);
      lu[1507] = a79;
      lu[1508] = a145;
      lu[1509] = a148;
      vd[31] = 1.0 / a31;
    }
    { // row 32
      double a32 = 1.0;
      a32 = fma(-r1delt, ws[1205], a32);
      a32 = fma(-r1delt, ws[1987], a32);
      double a107 = 0.0;
      a107 = fma(r1delt, ws[1197], a107);
      double a145 = 0.0;
      a145 = fma(-r1delt, ws[1988], a145);
      lu[1505] = a107;
      lu[1506] = a145;
      vd[32] = 1.0 / a32;
    }
    { // row 33
      double a33 = 1.0;
      a33 = fma(-r1delt, ws[1989], a33);
      a33 = fma(-r1delt, ws[1322], a33);
      double a52 = 0.0;
      a52 = fma(0.904 * r1delt, ws[1985], a52);
      double a148 = 0.0;
      a148 = fma(0.904 * r1delt, ws[1986], a148);
      a148 = fma(-r1delt, ws[1990], a148);
      lu[1503] = a52;
      lu[1504] = a148;
      vd[33] = 1.0 / a33;
    }
    { // row 34
      double a34 = 1.0;
      a34 = fma(-r1delt, ws[2027], a34);
      a34 = fma(-r1delt, ws[2134], a34);
      double a142 = 0.0;
      a142 = fma(-r1delt, ws[2133], a142);
      double a148 = 0.0;
      a148 = fma(-r1delt, ws[2028], a148);
      lu[1501] = a142;
      lu[1502] = a148;
      vd[34] = 1.0 / a34;
    }
    { // row 35
      double a35 = 1.0;
      a35 = fma(-r1delt, ws[2037], a35);
      a35 = fma(-r1delt, ws[2136], a35);
      double a142 = 0.0;
      a142 = fma(-r1delt, ws[2135], a142);
      double a148 = 0.0;
      a148 = fma(-r1delt, ws[2038], a148);
      lu[1499] = a142;
      lu[1500] = a148;
      vd[35] = 1.0 / a35;
    }
    { // row 36
      double a36 = 1.0;
      a36 = fma(-r1delt, ws[2039], a36);
      a36 = fma(-r1delt, ws[2138], a36);
      double a142 = 0.0;
      a142 = fma(-r1delt, ws[2137], a142);
      double a148 = 0.0;
      a148 = fma(-r1delt, ws[2040], a148);
      lu[1497] = a142;
      lu[1498] = a148;
      vd[36] = 1.0 / a36;
    }
    { // row 37
      double a37 = 1.0;
      a37 = fma(-r1delt, ws[1268], a37);
      a37 = fma(-r1delt, ws[2262], a37);
      a37 = fma(r1delt, ws[2262], a37);
      double a94 = 0.0;
      a94 = fma(-r1delt, ws[2261], a94);
      a94 = fma(r1delt, ws[2261], a94);
      double a110 = 0.0;
      a110 = fma(0.3 * r1delt, ws[2097], a110);
      a110 = fma(0.3 * r1delt, ws[2098], a110);
      lu[1495] = a94;
      lu[1496] = a110;
      vd[37] = 1.0 / a37;
    }
    { // row 38
      double a38 = 1.0;
      a38 = fma(-r1delt, ws[1296], a38);
      a38 = fma(-r1delt, ws[1297], a38);
      a38 = fma(-r1delt, ws[1298], a38);
      a38 = fma(-r1delt, ws[1299], a38);
      double a110 = 0.0;
      a110 = fma(r1delt, ws[2139], a110);
      double a144 = 0.0;
      a144 = fma(r1delt, ws[2140], a144);
      lu[1493] = a110;
      lu[1494] = a144;
      vd[38] = 1.0 / a38;
    }
    { // row 39
      double a17 = 0.0;
      a17 = fma(-r1delt, ws[2170], a17);
      double a39 = 1.0;
      a39 = fma(-r1delt, ws[1316], a39);
      a39 = fma(-r1delt, ws[2169], a39);
      double a40 = 0.0;
      a40 = fma(r1delt, ws[1314], a40);
      a17 = a17 * CHEM_LDLU(vd + 17);
      lu[5] = a17;
      a39 = fma(-a17, CHEM_LDLU(lu + 1529), a39);
      lu[1492] = a40;
      vd[39] = 1.0 / a39;
    }
    { // row 40
      double a40 = 1.0;
      a40 = fma(-r1delt, ws[1079], a40);
      a40 = fma(-r1delt, ws[1080], a40);
      a40 = fma(-r1delt, ws[1081], a40);
      a40 = fma(-r1delt, ws[1313], a40);
      a40 = fma(-r1delt, ws[1314], a40);
      double a144 = 0.0;
      a144 = fma(r1delt, ws[1794], a144);
      double a145 = 0.0;
      a145 = fma(r1delt, ws[1793], a145);
      lu[1490] = a144;
      lu[1491] = a145;
      vd[40] = 1.0 / a40;
    }
    { // row 41
      double a18 = 0.0;
      a18 = fma(-r1delt, ws[2172], a18);
      double a33 = 0.0;
      a33 = fma(r1delt, ws[1322], a33);
      double a41 = 1.0;
      a41 = fma(-r1delt, ws[2171], a41);
      a41 = fma(-r1delt, ws[1324], a41);
      double a52 = 0.0;
      double a148 = 0.0;
      a18 = a18 * CHEM_LDLU(vd + 18);
      lu[6] = a18;
      a41 = fma(-a18, CHEM_LDLU(lu + 1528), a41);
      a33 = a33 * CHEM_LDLU(vd + 33);
      lu[7] = a33;
      a52 = fma(-a33, CHEM_LDLU(lu + 1503), a52);
      a148 = fma(-a33, CHEM_LDLU(lu + 1504), a148);
      lu[1488] = a52;
      lu[1489] = a148;
      vd[41] = 1.0 / a41;
    }
    { // row 42
      double a42 = 1.0;
      a42 = fma(-r1delt, ws[1097], a42);
      a42 = fma(-r1delt, ws[1098], a42);
      double a139 = 0.0;
      a139 = fma(r1delt, ws[1815], a139);
      double a144 = 0.0;
      a144 = fma(r1delt, ws[1816], a144);
      lu[1486] = a139;
      lu[1487] = a144;
      vd[42] = 1.0 / a42;
    }
    { // row 43
      double a2 = 0.0;
      a2 = fma(0.907 * r1delt, ws[1335], a2);
      double a3 = 0.0;
      a3 = fma(0.925 * r1delt, ws[1336], a3);
      double a4 = 0.0;
      a4 = fma(0.943 * r1delt, ws[1337], a4);
      double a43 = 1.0;
      a2 = a2 * CHEM_LDLU(vd + 2);
      lu[8] = a2;
      a3 = a3 * CHEM_LDLU(vd + 3);
      lu[9] = a3;
      a4 = a4 * CHEM_LDLU(vd + 4);
      lu[10] = a4;
      vd[43] = 1.0 / a43;
    }
    { // row 44
      double a5 = 0.0;
      a5 = fma(0.5 * r1delt, ws[1338], a5);
      double a6 = 0.0;
      a6 = fma(0.5 * r1delt, ws[1339], a6);
      double a7 = 0.0;
      a7 = fma(1.5 * r1delt, ws[1340], a7);
      double a44 = 1.0;
      a5 = a5 * CHEM_LDLU(vd + 5);
      lu[11] = a5;
      a6 = a6 * CHEM_LDLU(vd + 6);
      lu[12] = a6;
      a7 = a7 * CHEM_LDLU(vd + 7);
      lu[13] = a7;
      vd[44] = 1.0 / a44;
    }
    { // row 45
      double a22 = 0.0;
      a22 = fma(1.25 * r1delt, ws[2185], a22);
      double a45 = 1.0;
      a45 = fma(-r1delt, ws[2187], a45);
      double a148 = 0.0;
      a148 = fma(1.25 * r1delt, ws[2186], a148);
      a148 = fma(-r1delt, ws[2188], a148);
      a22 = a22 * CHEM_LDLU(vd + 22);
      lu[14] = a22;
      a148 = fma(-a22, CHEM_LDLU(lu + 1523), a148);
      lu[1485] = a148;
      vd[45] = 1.0 / a45;
    }
    { // row 46
      double a23 = 0.0;
      a23 = fma(1.25 * r1delt, ws[2189], a23);
      double a46 = 1.0;
      a46 = fma(-r1delt, ws[2191], a46);
      double a148 = 0.0;
      a148 = fma(1.25 * r1delt, ws[2190], a148);
      a148 = fma(-r1delt, ws[2192], a148);
      a23 = a23 * CHEM_LDLU(vd + 23);
      lu[15] = a23;
      a148 = fma(-a23, CHEM_LDLU(lu + 1522), a148);
      lu[1484] = a148;
      vd[46] = 1.0 / a46;
    }
    { // row 47
      double a47 = 1.0;
      a47 = fma(-r1delt, ws[2203], a47);
      double a86 = 0.0;
      a86 = fma(0.0023 * r1delt, ws[2195], a86);
      double a148 = 0.0;
      a148 = fma(0.0023 * r1delt, ws[2196], a148);
      a148 = fma(-r1delt, ws[2204], a148);
      lu[1482] = a86;
      lu[1483] = a148;
      vd[47] = 1.0 / a47;
    }
    { // row 48
      double a48 = 1.0;
      a48 = fma(-r1delt, ws[2255], a48);
      a48 = fma(-r1delt, ws[2257], a48);
      double a142 = 0.0;
      a142 = fma(-r1delt, ws[2258], a142);
      double a148 = 0.0;
      a148 = fma(-r1delt, ws[2256], a148);
      lu[1480] = a142;
      lu[1481] = a148;
      vd[48] = 1.0 / a48;
    }
    { // row 49
      double a49 = 1.0;
      double a94 = 0.0;
      a94 = fma(0.5 * r1delt, ws[2259], a94);
      a94 = fma(0.5 * r1delt, ws[2265], a94);
      double a135 = 0.0;
      a135 = fma(0.5 * r1delt, ws[2260], a135);
      double a148 = 0.0;
      a148 = fma(0.5 * r1delt, ws[2266], a148);
      lu[1477] = a94;
      lu[1478] = a135;
      lu[1479] = a148;
      vd[49] = 1.0 / a49;
    }
    { // row 50
      double a50 = 1.0;
      double a63 = 0.0;
      a63 = fma(0.25 * r1delt, ws[2271], a63);
      a63 = fma(0.14 * r1delt, ws[2275], a63);
      double a142 = 0.0;
      a142 = fma(0.14 * r1delt, ws[2276], a142);
      double a148 = 0.0;
      a148 = fma(0.25 * r1delt, ws[2272], a148);
      lu[1474] = a63;
      lu[1475] = a142;
      lu[1476] = a148;
      vd[50] = 1.0 / a50;
    }
    { // row 51
      double a51 = 1.0;
      a51 = fma(-r1delt, ws[1999], a51);
      a51 = fma(0.104 * r1delt, ws[1999], a51);
      double a107 = 0.0;
      a107 = fma(0.1 * r1delt, ws[1967], a107);
      double a137 = 0.0;
      a137 = fma(0.1 * r1delt, ws[1968], a137);
      double a148 = 0.0;
      a148 = fma(-r1delt, ws[2000], a148);
      a148 = fma(0.104 * r1delt, ws[2000], a148);
      lu[1471] = a107;
      lu[1472] = a137;
      lu[1473] = a148;
      vd[51] = 1.0 / a51;
    }
    { // row 52
      double a52 = 1.0;
      a52 = fma(-r1delt, ws[1985], a52);
      double a107 = 0.0;
      a107 = fma(0.88 * r1delt, ws[1969], a107);
      double a147 = 0.0;
      a147 = fma(0.88 * r1delt, ws[1970], a147);
      double a148 = 0.0;
      a148 = fma(-r1delt, ws[1986], a148);
      lu[1468] = a107;
      lu[1469] = a147;
      lu[1470] = a148;
      vd[52] = 1.0 / a52;
    }
    { // row 53
      double a53 = 1.0;
      a53 = fma(-r1delt, ws[1091], a53);
      a53 = fma(-r1delt, ws[1092], a53);
      a53 = fma(-r1delt, ws[1809], a53);
      double a144 = 0.0;
      a144 = fma(r1delt, ws[1808], a144);
      double a147 = 0.0;
      a147 = fma(r1delt, ws[1807], a147);
      double a148 = 0.0;
      a148 = fma(-r1delt, ws[1810], a148);
      lu[1465] = a144;
      lu[1466] = a147;
      lu[1467] = a148;
      vd[53] = 1.0 / a53;
    }
    { // row 54
      double a54 = 1.0;
      a54 = fma(-r1delt, ws[1144], a54);
      a54 = fma(-r1delt, ws[1893], a54);
      a54 = fma(-r1delt, ws[1895], a54);
      double a137 = 0.0;
      a137 = fma(-r1delt, ws[1894], a137);
      double a141 = 0.0;
      a141 = fma(r1delt, ws[1891], a141);
      double a147 = 0.0;
      a147 = fma(r1delt, ws[1892], a147);
      a147 = fma(-r1delt, ws[1896], a147);
      lu[1462] = a137;
      lu[1463] = a141;
      lu[1464] = a147;
      vd[54] = 1.0 / a54;
    }
    { // row 55
      double a55 = 1.0;
      a55 = fma(-r1delt, ws[2073], a55);
      a55 = fma(-r1delt, ws[2075], a55);
      double a113 = 0.0;
      a113 = fma(0.732 * r1delt, ws[2049], a113);
      double a145 = 0.0;
      a145 = fma(-r1delt, ws[2076], a145);
      double a148 = 0.0;
      a148 = fma(0.732 * r1delt, ws[2050], a148);
      a148 = fma(-r1delt, ws[2074], a148);
      lu[1459] = a113;
      lu[1460] = a145;
      lu[1461] = a148;
      vd[55] = 1.0 / a55;
    }
    { // row 56
      double a56 = 1.0;
      a56 = fma(-r1delt, ws[1256], a56);
      a56 = fma(-r1delt, ws[2087], a56);
      double a117 = 0.0;
      a117 = fma(r1delt, ws[2079], a117);
      double a144 = 0.0;
      a144 = fma(r1delt, ws[2080], a144);
      double a148 = 0.0;
      a148 = fma(-r1delt, ws[2088], a148);
      lu[1456] = a117;
      lu[1457] = a144;
      lu[1458] = a148;
      vd[56] = 1.0 / a56;
    }
    { // row 57
      double a38 = 0.0;
      a38 = fma(r1delt, ws[1298], a38);
      a38 = fma(r1delt, ws[1299], a38);
      double a57 = 1.0;
      a57 = fma(-r1delt, ws[1269], a57);
      double a110 = 0.0;
      a110 = fma(r1delt, ws[2101], a110);
      double a144 = 0.0;
      double a147 = 0.0;
      a147 = fma(r1delt, ws[2102], a147);
      a38 = a38 * CHEM_LDLU(vd + 38);
      lu[16] = a38;
      a110 = fma(-a38, CHEM_LDLU(lu + 1493), a110);
      a144 = fma(-a38, CHEM_LDLU(lu + 1494), a144);
      lu[1453] = a110;
      lu[1454] = a144;
      lu[1455] = a147;
      vd[57] = 1.0 / a57;
    }
    { // row 58
      double a58 = 1.0;
      a58 = fma(-r1delt, ws[2153], a58);
      a58 = fma(-r1delt, ws[2155], a58);
      a58 = fma(-r1delt, ws[2157], a58);
      double a135 = 0.0;
      a135 = fma(-r1delt, ws[2154], a135);
      double a145 = 0.0;
      a145 = fma(-r1delt, ws[2158], a145);
      double a148 = 0.0;
      a148 = fma(-r1delt, ws[2156], a148);
      lu[1450] = a135;
      lu[1451] = a145;
      lu[1452] = a148;
      vd[58] = 1.0 / a58;
    }
    { // row 59
      double a58 = 0.0;
      a58 = fma(r1delt, ws[2153], a58);
      a58 = fma(r1delt, ws[2155], a58);
      a58 = fma(r1delt, ws[2157], a58);
      double a59 = 1.0;
      double a135 = 0.0;
      a135 = fma(r1delt, ws[2154], a135);
      double a145 = 0.0;
      a145 = fma(r1delt, ws[2158], a145);
      double a148 = 0.0;
      a148 = fma(r1delt, ws[2156], a148);
      a58 = a58 * CHEM_LDLU(vd + 58);
      lu[17] = a58;
      a135 = fma(-a58, CHEM_LDLU(lu + 1450), a135);
      a145 = fma(-a58, CHEM_LDLU(lu + 1451), a145);
      a148 = fma(-a58, CHEM_LDLU(lu + 1452), a148);
      lu[1447] = a135;
      lu[1448] = a145;
      lu[1449] = a148;
      vd[59] = 1.0 / a59;
    }
    { // row 60
      double a15 = 0.0;
      a15 = fma(-r1delt, ws[2166], a15);
      double a16 = 0.0;
      a16 = fma(-r1delt, ws[2168], a16);
      double a40 = 0.0;
      a40 = fma(r1delt, ws[1313], a40);
      double a60 = 1.0;
      a60 = fma(-r1delt, ws[1315], a60);
      a60 = fma(-r1delt, ws[2165], a60);
      a60 = fma(-r1delt, ws[2167], a60);
      double a144 = 0.0;
      double a145 = 0.0;
      a15 = a15 * CHEM_LDLU(vd + 15);
      lu[18] = a15;
      a60 = fma(-a15, CHEM_LDLU(lu + 1531), a60);
      a16 = a16 * CHEM_LDLU(vd + 16);
      lu[19] = a16;
      a60 = fma(-a16, CHEM_LDLU(lu + 1530), a60);
      a40 = a40 * CHEM_LDLU(vd + 40);
      lu[20] = a40;
      a144 = fma(-a40, CHEM_LDLU(lu + 1490), a144);
      a145 = fma(-a40, CHEM_LDLU(lu + 1491), a145);
      lu[1445] = a144;
      lu[1446] = a145;
      vd[60] = 1.0 / a60;
    }
    { // row 61
      double a61 = 1.0;
      a61 = fma(-r1delt, ws[1105], a61);
      a61 = fma(-r1delt, ws[1106], a61);
      a61 = fma(-r1delt, ws[2089], a61);
      double a128 = 0.0;
      a128 = fma(r1delt, ws[1827], a128);
      double a144 = 0.0;
      a144 = fma(r1delt, ws[1828], a144);
      double a148 = 0.0;
      a148 = fma(-r1delt, ws[2090], a148);
      lu[1442] = a128;
      lu[1443] = a144;
      lu[1444] = a148;
      vd[61] = 1.0 / a61;
    }
}
__device__ __noinline__ void gear_pdecomp_s1_0_1(double* __restrict__ ws, double r1delt)
{
    double* __restrict__ lu = ws + 2426;
    double* __restrict__ vd = ws + 4116;
    { // row 62
      double a62 = 1.0;
      a62 = fma(-r1delt, ws[1265], a62);
      a62 = fma(-r1delt, ws[1266], a62);
      double a132 = 0.0;
      a132 = fma(r1delt, ws[1933], a132);
      a132 = fma(r1delt, ws[2108], a132);
      double a142 = 0.0;
      a142 = fma(r1delt, ws[2107], a142);
      double a148 = 0.0;
      a148 = fma(r1delt, ws[1934], a148);
      lu[1439] = a132;
      lu[1440] = a142;
      lu[1441] = a148;
      vd[62] = 1.0 / a62;
    }
    { // row 63
      double a63 = 1.0;
      a63 = fma(-r1delt, ws[2269], a63);
      a63 = fma(-r1delt, ws[2271], a63);
      a63 = fma(-r1delt, ws[2273], a63);
      a63 = fma(-r1delt, ws[2275], a63);
      double a142 = 0.0;
      a142 = fma(-r1delt, ws[2276], a142);
      double a145 = 0.0;
      a145 = fma(-r1delt, ws[2274], a145);
      double a148 = 0.0;
      a148 = fma(-r1delt, ws[2270], a148);
      a148 = fma(-r1delt, ws[2272], a148);
      lu[1436] = a142;
      lu[1437] = a145;
      lu[1438] = a148;
      vd[63] = 1.0 / a63;
    }
    { // row 64
      double a64 = 1.0;
      a64 = fma(-r1delt, ws[2001], a64);
      a64 = fma(-r1delt, ws[2003], a64);
      a64 = fma(-r1delt, ws[2005], a64);
      a64 = fma(-r1delt, ws[2007], a64);
      double a130 = 0.0;
      a130 = fma(-r1delt, ws[2002], a130);
      double a135 = 0.0;
      a135 = fma(-r1delt, ws[2006], a135);
      double a145 = 0.0;
      a145 = fma(-r1delt, ws[2008], a145);
      double a148 = 0.0;
      a148 = fma(-r1delt, ws[2004], a148);
      lu[1432] = a130;
      lu[1433] = a135;
      lu[1434] = a145;
      lu[1435] = a148;
      vd[64] = 1.0 / a64;
    }
    { // row 65
      double a64 = 0.0;
      a64 = fma(r1delt, ws[2001], a64);
      a64 = fma(r1delt, ws[2003], a64);
      a64 = fma(r1delt, ws[2005], a64);
      double a65 = 1.0;
      double a66 = 0.0;
      a66 = fma(r1delt, ws[2009], a66);
      a66 = fma(r1delt, ws[2011], a66);
      a66 = fma(r1delt, ws[2013], a66);
      double a130 = 0.0;
      a130 = fma(r1delt, ws[2002], a130);
      a130 = fma(r1delt, ws[2010], a130);
      double a135 = 0.0;
      a135 = fma(r1delt, ws[2006], a135);
      a135 = fma(r1delt, ws[2014], a135);
      double a145 = 0.0;
      double a148 = 0.0;
      a148 = fma(r1delt, ws[2004], a148);
      a148 = fma(r1delt, ws[2012], a148);
      a64 = a64 * CHEM_LDLU(vd + 64);
      lu[21] = a64;
      a130 = fma(-a64, CHEM_LDLU(lu + 1432), a130);
      a135 = fma(-a64, CHEM_LDLU(lu + 1433), a135);
      a145 = fma(-a64, CHEM_LDLU(lu + 1434), a145);
      a148 = fma(-a64, CHEM_LDLU(lu + 1435), a148);
      lu[1427] = a66;
      lu[1428] = a130;
      lu[1429] = a135;
      lu[1430] = a145;
      lu[1431] = a148;
      vd[65] = 1.0 / a65;
    }
    { // row 66
      double a66 = 1.0;
      a66 = fma(-r1delt, ws[2009], a66);
      a66 = fma(-r1delt, ws[2011], a66);
      a66 = fma(-r1delt, ws[2013], a66);
      a66 = fma(-r1delt, ws[2015], a66);
      double a130 = 0.0;
      a130 = fma(-r1delt, ws[2010], a130);
      double a135 = 0.0;
      a135 = fma(-r1delt, ws[2014], a135);
      double a145 = 0.0;
      a145 = fma(-r1delt, ws[2016], a145);
      double a148 = 0.0;
      a148 = fma(-r1delt, ws[2012], a148);
      lu[1423] = a130;
      lu[1424] = a135;
      lu[1425] = a145;
      lu[1426] = a148;
      vd[66] = 1.0 / a66;
    }
    { // row 67
      double a12 = 0.0;
      a12 = fma(r1delt, ws[2017], a12);
      double a67 = 1.0;
      a67 = fma(-r1delt, ws[2149], a67);
      a67 = fma(-r1delt, ws[2151], a67);
      double a137 = 0.0;
      a137 = fma(-r1delt, ws[2150], a137);
      double a147 = 0.0;
      a147 = fma(-r1delt, ws[2152], a147);
      double a148 = 0.0;
      a148 = fma(r1delt, ws[2018], a148);
      a12 = a12 * CHEM_LDLU(vd + 12);
      lu[22] = a12;
      a148 = fma(-a12, CHEM_LDLU(lu + 1534), a148);
      lu[1420] = a137;
      lu[1421] = a147;
      lu[1422] = a148;
      vd[67] = 1.0 / a67;
    }
    { // row 68
      double a68 = 1.0;
      a68 = fma(-r1delt, ws[2057], a68);
      a68 = fma(-r1delt, ws[2059], a68);
      a68 = fma(-r1delt, ws[1243], a68);
      double a104 = 0.0;
      a104 = fma(r1delt, ws[2053], a104);
      double a144 = 0.0;
      a144 = fma(r1delt, ws[2054], a144);
      double a145 = 0.0;
      a145 = fma(-r1delt, ws[2060], a145);
      double a148 = 0.0;
      a148 = fma(-r1delt, ws[2058], a148);
      lu[1416] = a104;
      lu[1417] = a144;
      lu[1418] = a145;
      lu[1419] = a148;
      vd[68] = 1.0 / a68;
    }
    { // row 69
      double a63 = 0.0;
      a63 = fma(r1delt, ws[2269], a63);
      a63 = fma(0.75 * r1delt, ws[2271], a63);
      a63 = fma(r1delt, ws[2273], a63);
      a63 = fma(0.86 * r1delt, ws[2275], a63);
      double a69 = 1.0;
      a69 = fma(-r1delt, ws[1811], a69);
      double a142 = 0.0;
      a142 = fma(0.86 * r1delt, ws[2276], a142);
      double a145 = 0.0;
      a145 = fma(r1delt, ws[2274], a145);
      double a148 = 0.0;
      a148 = fma(-r1delt, ws[1812], a148);
      a148 = fma(r1delt, ws[2270], a148);
      a148 = fma(0.75 * r1delt, ws[2272], a148);
      a63 = a63 * CHEM_LDLU(vd + 63);
      lu[23] = a63;
      a142 = fma(-a63, CHEM_LDLU(lu + 1436), a142);
      a145 = fma(-a63, CHEM_LDLU(lu + 1437), a145);
      a148 = fma(-a63, CHEM_LDLU(lu + 1438), a148);
      lu[1413] = a142;
      lu[1414] = a145;
      lu[1415] = a148;
      vd[69] = 1.0 / a69;
    }
    { // row 70
      double a67 = 0.0;
      a67 = fma(0.146 * r1delt, ws[2151], a67);
      double a70 = 1.0;
      double a78 = 0.0;
      a78 = fma(0.193 * r1delt, ws[2147], a78);
      double a80 = 0.0;
      a80 = fma(0.473 * r1delt, ws[2161], a80);
      double a92 = 0.0;
      a92 = fma(0.14 * r1delt, ws[2143], a92);
      double a137 = 0.0;
      double a147 = 0.0;
      a147 = fma(0.14 * r1delt, ws[2144], a147);
      a147 = fma(0.193 * r1delt, ws[2148], a147);
      a147 = fma(0.146 * r1delt, ws[2152], a147);
      a147 = fma(0.473 * r1delt, ws[2162], a147);
      double a148 = 0.0;
      a67 = a67 * CHEM_LDLU(vd + 67);
      lu[24] = a67;
      a137 = fma(-a67, CHEM_LDLU(lu + 1420), a137);
      a147 = fma(-a67, CHEM_LDLU(lu + 1421), a147);
      a148 = fma(-a67, CHEM_LDLU(lu + 1422), a148);
      lu[1407] = a78;
      lu[1408] = a80;
      lu[1409] = a92;
      lu[1410] = a137;
      lu[1411] = a147;
      lu[1412] = a148;
      vd[70] = 1.0 / a70;
    }
    { // row 71
      double a54 = 0.0;
      a54 = fma(0.5 * r1delt, ws[1895], a54);
      double a71 = 1.0;
      a71 = fma(-r1delt, ws[1873], a71);
      a71 = fma(-r1delt, ws[1130], a71);
      double a137 = 0.0;
      double a138 = 0.0;
      a138 = fma(0.9 * r1delt, ws[1843], a138);
      double a141 = 0.0;
      double a147 = 0.0;
      a147 = fma(0.9 * r1delt, ws[1844], a147);
      a147 = fma(0.5 * r1delt, ws[1896], a147);
      double a148 = 0.0;
      a148 = fma(-r1delt, ws[1874], a148);
      a54 = a54 * CHEM_LDLU(vd + 54);
      lu[25] = a54;
      a137 = fma(-a54, CHEM_LDLU(lu + 1462), a137);
      a141 = fma(-a54, CHEM_LDLU(lu + 1463), a141);
      a147 = fma(-a54, CHEM_LDLU(lu + 1464), a147);
      lu[1402] = a137;
      lu[1403] = a138;
      lu[1404] = a141;
      lu[1405] = a147;
      lu[1406] = a148;
      vd[71] = 1.0 / a71;
    }
    { // row 72
      double a72 = 1.0;
      a72 = fma(-r1delt, ws[2201], a72);
      a72 = fma(0.1043 * r1delt, ws[2201], a72);
      double a86 = 0.0;
      a86 = fma(0.0026 * r1delt, ws[2195], a86);
      double a87 = 0.0;
      a87 = fma(0.0035 * r1delt, ws[2197], a87);
      double a88 = 0.0;
      a88 = fma(0.0005 * r1delt, ws[2199], a88);
      double a148 = 0.0;
      a148 = fma(0.0026 * r1delt, ws[2196], a148);
      a148 = fma(0.0035 * r1delt, ws[2198], a148);
      a148 = fma(0.0005 * r1delt, ws[2200], a148);
      a148 = fma(-r1delt, ws[2202], a148);
      a148 = fma(0.1043 * r1delt, ws[2202], a148);
      lu[1398] = a86;
      lu[1399] = a87;
      lu[1400] = a88;
      lu[1401] = a148;
      vd[72] = 1.0 / a72;
    }
    { // row 73
      double a73 = 1.0;
      a73 = fma(-r1delt, ws[2215], a73);
      a73 = fma(-r1delt, ws[2217], a73);
      a73 = fma(-r1delt, ws[2219], a73);
      a73 = fma(-r1delt, ws[1359], a73);
      a73 = fma(-r1delt, ws[1360], a73);
      a73 = fma(-r1delt, ws[2221], a73);
      double a130 = 0.0;
      a130 = fma(-r1delt, ws[2220], a130);
      double a142 = 0.0;
      a142 = fma(-r1delt, ws[2222], a142);
      double a145 = 0.0;
      a145 = fma(-r1delt, ws[2218], a145);
      double a148 = 0.0;
      a148 = fma(-r1delt, ws[2216], a148);
      lu[1394] = a130;
      lu[1395] = a142;
      lu[1396] = a145;
      lu[1397] = a148;
      vd[73] = 1.0 / a73;
    }
    { // row 74
      double a74 = 1.0;
      a74 = fma(-r1delt, ws[2223], a74);
      a74 = fma(-r1delt, ws[2225], a74);
      a74 = fma(-r1delt, ws[2227], a74);
      a74 = fma(-r1delt, ws[1365], a74);
      a74 = fma(-r1delt, ws[2229], a74);
      double a130 = 0.0;
      a130 = fma(-r1delt, ws[2228], a130);
      double a142 = 0.0;
      a142 = fma(-r1delt, ws[2230], a142);
      double a145 = 0.0;
      a145 = fma(-r1delt, ws[2226], a145);
      double a148 = 0.0;
      a148 = fma(-r1delt, ws[2224], a148);
      lu[1390] = a130;
      lu[1391] = a142;
      lu[1392] = a145;
      lu[1393] = a148;
      vd[74] = 1.0 / a74;
    }
    { // row 75
      double a75 = 1.0;
      a75 = fma(-r1delt, ws[2231], a75);
      a75 = fma(-r1delt, ws[2233], a75);
      a75 = fma(-r1delt, ws[2235], a75);
      a75 = fma(-r1delt, ws[2237], a75);
      double a135 = 0.0;
      a135 = fma(-r1delt, ws[2234], a135);
      double a142 = 0.0;
      a142 = fma(-r1delt, ws[2238], a142);
      double a145 = 0.0;
      a145 = fma(-r1delt, ws[2236], a145);
      double a148 = 0.0;
      a148 = fma(-r1delt, ws[2232], a148);
      lu[1386] = a135;
      lu[1387] = a142;
      lu[1388] = a145;
      lu[1389] = a148;
      vd[75] = 1.0 / a75;
    }
    { // row 76
      double a76 = 1.0;
      a76 = fma(-r1delt, ws[2239], a76);
      a76 = fma(-r1delt, ws[2241], a76);
      a76 = fma(-r1delt, ws[2243], a76);
      a76 = fma(-r1delt, ws[1374], a76);
      a76 = fma(-r1delt, ws[2245], a76);
      double a135 = 0.0;
      a135 = fma(-r1delt, ws[2242], a135);
      double a142 = 0.0;
      a142 = fma(-r1delt, ws[2246], a142);
      double a145 = 0.0;
      a145 = fma(-r1delt, ws[2244], a145);
      double a148 = 0.0;
      a148 = fma(-r1delt, ws[2240], a148);
      lu[1382] = a135;
      lu[1383] = a142;
      lu[1384] = a145;
      lu[1385] = a148;
      vd[76] = 1.0 / a76;
    }
    { // row 77
      double a68 = 0.0;
      a68 = fma(r1delt, ws[1243], a68);
      double a77 = 1.0;
      a77 = fma(-r1delt, ws[1799], a77);
      a77 = fma(-r1delt, ws[1799], a77);
      a77 = fma(-r1delt, ws[1800], a77);
      a77 = fma(-r1delt, ws[1800], a77);
      a77 = fma(-r1delt, ws[1085], a77);
      a77 = fma(-r1delt, ws[1801], a77);
      double a104 = 0.0;
      double a137 = 0.0;
      a137 = fma(r1delt, ws[1795], a137);
      a137 = fma(2.0 * r1delt, ws[1797], a137);
      double a144 = 0.0;
      a144 = fma(2.0 * r1delt, ws[1798], a144);
      a144 = fma(0.5 * r1delt, ws[1320], a144);
      double a145 = 0.0;
      double a148 = 0.0;
      a148 = fma(r1delt, ws[1796], a148);
      a148 = fma(-r1delt, ws[1802], a148);
      a68 = a68 * CHEM_LDLU(vd + 68);
      lu[26] = a68;
      a104 = fma(-a68, CHEM_LDLU(lu + 1416), a104);
      a144 = fma(-a68, CHEM_LDLU(lu + 1417), a144);
      a145 = fma(-a68, CHEM_LDLU(lu + 1418), a145);
      a148 = fma(-a68, CHEM_LDLU(lu + 1419), a148);
      lu[1377] = a104;
      lu[1378] = a137;
      lu[1379] = a144;
      lu[1380] = a145;
      lu[1381] = a148;
      vd[77] = 1.0 / a77;
    }
    { // row 78
      double a35 = 0.0;
      a35 = fma(r1delt, ws[2037], a35);
      a35 = fma(r1delt, ws[2136], a35);
      double a78 = 1.0;
      a78 = fma(-r1delt, ws[2145], a78);
      a78 = fma(-r1delt, ws[2147], a78);
      double a137 = 0.0;
      a137 = fma(-r1delt, ws[2146], a137);
      double a142 = 0.0;
      a142 = fma(r1delt, ws[2135], a142);
      double a147 = 0.0;
      a147 = fma(-r1delt, ws[2148], a147);
      double a148 = 0.0;
      a148 = fma(r1delt, ws[2038], a148);
      a35 = a35 * CHEM_LDLU(vd + 35);
      lu[27] = a35;
      a142 = fma(-a35, CHEM_LDLU(lu + 1499), a142);
      a148 = fma(-a35, CHEM_LDLU(lu + 1500), a148);
      lu[1373] = a137;
      lu[1374] = a142;
      lu[1375] = a147;
      lu[1376] = a148;
      vd[78] = 1.0 / a78;
    }
    { // row 79
      double a79 = 1.0;
      a79 = fma(-r1delt, ws[1963], a79);
      a79 = fma(-r1delt, ws[1965], a79);
      a79 = fma(-r1delt, ws[1975], a79);
      a79 = fma(-r1delt, ws[1977], a79);
      a79 = fma(-r1delt, ws[2120], a79);
      double a130 = 0.0;
      a130 = fma(-r1delt, ws[1966], a130);
      double a135 = 0.0;
      a135 = fma(-r1delt, ws[1976], a135);
      double a142 = 0.0;
      a142 = fma(-r1delt, ws[2119], a142);
      double a145 = 0.0;
      a145 = fma(-r1delt, ws[1978], a145);
      double a148 = 0.0;
      a148 = fma(-r1delt, ws[1964], a148);
      lu[1368] = a130;
      lu[1369] = a135;
      lu[1370] = a142;
      lu[1371] = a145;
      lu[1372] = a148;
      vd[79] = 1.0 / a79;
    }
    { // row 80
      double a36 = 0.0;
      a36 = fma(r1delt, ws[2039], a36);
      a36 = fma(r1delt, ws[2138], a36);
      double a80 = 1.0;
      a80 = fma(-r1delt, ws[2159], a80);
      a80 = fma(-r1delt, ws[2161], a80);
      double a137 = 0.0;
      a137 = fma(-r1delt, ws[2160], a137);
      double a142 = 0.0;
      a142 = fma(r1delt, ws[2137], a142);
      double a147 = 0.0;
      a147 = fma(-r1delt, ws[2162], a147);
      double a148 = 0.0;
      a148 = fma(r1delt, ws[2040], a148);
      a36 = a36 * CHEM_LDLU(vd + 36);
      lu[28] = a36;
      a142 = fma(-a36, CHEM_LDLU(lu + 1497), a142);
      a148 = fma(-a36, CHEM_LDLU(lu + 1498), a148);
      lu[1364] = a137;
      lu[1365] = a142;
      lu[1366] = a147;
      lu[1367] = a148;
      vd[80] = 1.0 / a80;
    }
    { // row 81
      double a15 = 0.0;
      a15 = fma(r1delt, ws[2166], a15);
      double a16 = 0.0;
      a16 = fma(r1delt, ws[2168], a16);
      double a17 = 0.0;
      a17 = fma(r1delt, ws[2170], a17);
      double a39 = 0.0;
      a39 = fma(r1delt, ws[2169], a39);
      double a40 = 0.0;
      double a60 = 0.0;
      a60 = fma(r1delt, ws[2165], a60);
      a60 = fma(r1delt, ws[2167], a60);
      double a81 = 1.0;
      a81 = fma(-r1delt, ws[1294], a81);
      double a144 = 0.0;
      double a145 = 0.0;
      a15 = a15 * CHEM_LDLU(vd + 15);
      lu[29] = a15;
      a60 = fma(-a15, CHEM_LDLU(lu + 1531), a60);
      a16 = a16 * CHEM_LDLU(vd + 16);
      lu[30] = a16;
      a60 = fma(-a16, CHEM_LDLU(lu + 1530), a60);
      a17 = a17 * CHEM_LDLU(vd + 17);
      lu[31] = a17;
      a39 = fma(-a17, CHEM_LDLU(lu + 1529), a39);
      a39 = a39 * CHEM_LDLU(vd + 39);
      lu[32] = a39;
      a40 = fma(-a39, CHEM_LDLU(lu + 1492), a40);
      a40 = a40 * CHEM_LDLU(vd + 40);
      lu[33] = a40;
      a144 = fma(-a40, CHEM_LDLU(lu + 1490), a144);
      a145 = fma(-a40, CHEM_LDLU(lu + 1491), a145);
      a60 = a60 * CHEM_LDLU(vd + 60);
      lu[34] = a60;
      a144 = fma(-a60, CHEM_LDLU(lu + 1445), a144);
      a145 = fma(-a60, CHEM_LDLU(lu + 1446), a145);
      lu[1362] = a144;
      lu[1363] = a145;
      vd[81] = 1.0 / a81;
    }
    { // row 82
      double a14 = 0.0;
      a14 = fma(0.052 * r1delt, ws[2163], a14);
      double a78 = 0.0;
      a78 = fma(0.023 * r1delt, ws[2145], a78);
      double a80 = 0.0;
      a80 = fma(0.225 * r1delt, ws[2159], a80);
      double a82 = 1.0;
      double a92 = 0.0;
      a92 = fma(0.051 * r1delt, ws[2141], a92);
      double a137 = 0.0;
      a137 = fma(0.051 * r1delt, ws[2142], a137);
      a137 = fma(0.023 * r1delt, ws[2146], a137);
      a137 = fma(0.225 * r1delt, ws[2160], a137);
      double a142 = 0.0;
      double a147 = 0.0;
      double a148 = 0.0;
      a148 = fma(0.052 * r1delt, ws[2164], a148);
      a14 = a14 * CHEM_LDLU(vd + 14);
      lu[35] = a14;
      a148 = fma(-a14, CHEM_LDLU(lu + 1532), a148);
      a78 = a78 * CHEM_LDLU(vd + 78);
      lu[36] = a78;
      a137 = fma(-a78, CHEM_LDLU(lu + 1373), a137);
      a142 = fma(-a78, CHEM_LDLU(lu + 1374), a142);
      a147 = fma(-a78, CHEM_LDLU(lu + 1375), a147);
      a148 = fma(-a78, CHEM_LDLU(lu + 1376), a148);
      a80 = a80 * CHEM_LDLU(vd + 80);
      lu[37] = a80;
      a137 = fma(-a80, CHEM_LDLU(lu + 1364), a137);
      a142 = fma(-a80, CHEM_LDLU(lu + 1365), a142);
      a147 = fma(-a80, CHEM_LDLU(lu + 1366), a147);
      a148 = fma(-a80, CHEM_LDLU(lu + 1367), a148);
      lu[1357] = a92;
      lu[1358] = a137;
      lu[1359] = a142;
      lu[1360] = a147;
      lu[1361] = a148;
      vd[82] = 1.0 / a82;
    }
    { // row 83
      double a83 = 1.0;
      a83 = fma(-r1delt, ws[1939], a83);
      a83 = fma(-r1delt, ws[1941], a83);
      a83 = fma(-r1delt, ws[1943], a83);
      a83 = fma(-r1delt, ws[1945], a83);
      a83 = fma(-r1delt, ws[2114], a83);
      double a130 = 0.0;
      a130 = fma(-r1delt, ws[1940], a130);
      double a135 = 0.0;
      a135 = fma(-r1delt, ws[1944], a135);
      double a142 = 0.0;
      a142 = fma(-r1delt, ws[2113], a142);
      double a145 = 0.0;
      a145 = fma(-r1delt, ws[1946], a145);
      double a148 = 0.0;
      a148 = fma(-r1delt, ws[1942], a148);
      lu[1352] = a130;
      lu[1353] = a135;
      lu[1354] = a142;
      lu[1355] = a145;
      lu[1356] = a148;
      vd[83] = 1.0 / a83;
    }
    { // row 84
      double a84 = 1.0;
      a84 = fma(-r1delt, ws[1883], a84);
      double a117 = 0.0;
      a117 = fma(0.37 * r1delt, ws[2081], a117);
      double a128 = 0.0;
      a128 = fma(0.37 * r1delt, ws[1829], a128);
      double a139 = 0.0;
      a139 = fma(0.37 * r1delt, ws[1817], a139);
      double a147 = 0.0;
      a147 = fma(0.37 * r1delt, ws[1818], a147);
      a147 = fma(0.37 * r1delt, ws[1830], a147);
      a147 = fma(0.37 * r1delt, ws[2082], a147);
      double a148 = 0.0;
      a148 = fma(-r1delt, ws[1884], a148);
      lu[1347] = a117;
      lu[1348] = a128;
      lu[1349] = a139;
      lu[1350] = a147;
      lu[1351] = a148;
      vd[84] = 1.0 / a84;
    }
    { // row 85
      double a85 = 1.0;
      a85 = fma(-r1delt, ws[1925], a85);
      a85 = fma(-r1delt, ws[2128], a85);
      double a120 = 0.0;
      a120 = fma(0.15 * r1delt, ws[1156], a120);
      double a138 = 0.0;
      a138 = fma(0.315 * r1delt, ws[1847], a138);
      double a142 = 0.0;
      a142 = fma(-r1delt, ws[2127], a142);
      double a146 = 0.0;
      a146 = fma(0.315 * r1delt, ws[1848], a146);
      double a148 = 0.0;
      a148 = fma(-r1delt, ws[1926], a148);
      lu[1342] = a120;
      lu[1343] = a138;
      lu[1344] = a142;
      lu[1345] = a146;
      lu[1346] = a148;
      vd[85] = 1.0 / a85;
    }
    { // row 86
      double a47 = 0.0;
      a47 = fma(0.2412 * r1delt, ws[2203], a47);
      double a72 = 0.0;
      a72 = fma(0.2181 * r1delt, ws[2201], a72);
      double a86 = 1.0;
      a86 = fma(-r1delt, ws[2195], a86);
      a86 = fma(0.4857 * r1delt, ws[2195], a86);
      double a87 = 0.0;
      a87 = fma(0.3003 * r1delt, ws[2197], a87);
      double a88 = 0.0;
      a88 = fma(0.3856 * r1delt, ws[2199], a88);
      double a148 = 0.0;
      a148 = fma(-r1delt, ws[2196], a148);
      a148 = fma(0.4857 * r1delt, ws[2196], a148);
      a148 = fma(0.3003 * r1delt, ws[2198], a148);
      a148 = fma(0.3856 * r1delt, ws[2200], a148);
      a148 = fma(0.2181 * r1delt, ws[2202], a148);
      a148 = fma(0.2412 * r1delt, ws[2204], a148);
      a47 = a47 * CHEM_LDLU(vd + 47);
      lu[38] = a47;
      a86 = fma(-a47, CHEM_LDLU(lu + 1482), a86);
      a148 = fma(-a47, CHEM_LDLU(lu + 1483), a148);
      a72 = a72 * CHEM_LDLU(vd + 72);
      lu[39] = a72;
      a86 = fma(-a72, CHEM_LDLU(lu + 1398), a86);
      a87 = fma(-a72, CHEM_LDLU(lu + 1399), a87);
      a88 = fma(-a72, CHEM_LDLU(lu + 1400), a88);
      a148 = fma(-a72, CHEM_LDLU(lu + 1401), a148);
      lu[1339] = a87;
      lu[1340] = a88;
      lu[1341] = a148;
      vd[86] = 1.0 / a86;
    }
}
__device__ __noinline__ void gear_pdecomp_s1_0_2(double* __restrict__ ws, double r1delt)
{
    double* __restrict__ lu = ws + 2426;
    double* __restrict__ vd = ws + 4116;
    { // row 87
      double a47 = 0.0;
      a47 = fma(0.2089 * r1delt, ws[2203], a47);
      double a72 = 0.0;
      a72 = fma(0.3063 * r1delt, ws[2201], a72);
      double a86 = 0.0;
      a86 = fma(0.0062 * r1delt, ws[2195], a86);
      double a87 = 1.0;
      a87 = fma(-r1delt, ws[2197], a87);
      a87 = fma(0.2862 * r1delt, ws[2197], a87);
      double a88 = 0.0;
      a88 = fma(0.095 * r1delt, ws[2199], a88);
      double a148 = 0.0;
      a148 = fma(0.0062 * r1delt, ws[2196], a148);
      a148 = fma(-r1delt, ws[2198], a148);
      a148 = fma(0.2862 * r1delt, ws[2198], a148);
      a148 = fma(0.095 * r1delt, ws[2200], a148);
      a148 = fma(0.3063 * r1delt, ws[2202], a148);
      a148 = fma(0.2089 * r1delt, ws[2204], a148);
      a47 = a47 * CHEM_LDLU(vd + 47);
      lu[40] = a47;
      a86 = fma(-a47, CHEM_LDLU(lu + 1482), a86);
      a148 = fma(-a47, CHEM_LDLU(lu + 1483), a148);
      a72 = a72 * CHEM_LDLU(vd + 72);
      lu[41] = a72;
      a86 = fma(-a72, CHEM_LDLU(lu + 1398), a86);
      a87 = fma(-a72, CHEM_LDLU(lu + 1399), a87);
      a88 = fma(-a72, CHEM_LDLU(lu + 1400), a88);
      a148 = fma(-a72, CHEM_LDLU(lu + 1401), a148);
      a86 = a86 * CHEM_LDLU(vd + 86);
      lu[42] = a86;
      a87 = fma(-a86, CHEM_LDLU(lu + 1339), a87);
      a88 = fma(-a86, CHEM_LDLU(lu + 1340), a88);
      a148 = fma(-a86, CHEM_LDLU(lu + 1341), a148);
      lu[1337] = a88;
      lu[1338] = a148;
      vd[87] = 1.0 / a87;
    }
    { // row 88
      double a47 = 0.0;
      a47 = fma(0.3 * r1delt, ws[2203], a47);
      double a72 = 0.0;
      a72 = fma(0.0153 * r1delt, ws[2201], a72);
      double a86 = 0.0;
      a86 = fma(0.0025 * r1delt, ws[2195], a86);
      double a87 = 0.0;
      a87 = fma(0.0041 * r1delt, ws[2197], a87);
      double a88 = 1.0;
      a88 = fma(-r1delt, ws[2199], a88);
      a88 = fma(0.1373 * r1delt, ws[2199], a88);
      double a148 = 0.0;
      a148 = fma(0.0025 * r1delt, ws[2196], a148);
      a148 = fma(0.0041 * r1delt, ws[2198], a148);
      a148 = fma(-r1delt, ws[2200], a148);
      a148 = fma(0.1373 * r1delt, ws[2200], a148);
      a148 = fma(0.0153 * r1delt, ws[2202], a148);
      a148 = fma(0.3 * r1delt, ws[2204], a148);
      a47 = a47 * CHEM_LDLU(vd + 47);
      lu[43] = a47;
      a86 = fma(-a47, CHEM_LDLU(lu + 1482), a86);
      a148 = fma(-a47, CHEM_LDLU(lu + 1483), a148);
      a72 = a72 * CHEM_LDLU(vd + 72);
      lu[44] = a72;
      a86 = fma(-a72, CHEM_LDLU(lu + 1398), a86);
      a87 = fma(-a72, CHEM_LDLU(lu + 1399), a87);
      a88 = fma(-a72, CHEM_LDLU(lu + 1400), a88);
      a148 = fma(-a72, CHEM_LDLU(lu + 1401), a148);
      a86 = a86 * CHEM_LDLU(vd + 86);
      lu[45] = a86;
      a87 = fma(-a86, CHEM_LDLU(lu + 1339), a87);
      a88 = fma(-a86, CHEM_LDLU(lu + 1340), a88);
      a148 = fma(-a86, CHEM_LDLU(lu + 1341), a148);
      a87 = a87 * CHEM_LDLU(vd + 87);
      lu[46] = a87;
      a88 = fma(-a87, CHEM_LDLU(lu + 1337), a88);
      a148 = fma(-a87, CHEM_LDLU(lu + 1338), a148);
      lu[1336] = a148;
      vd[88] = 1.0 / a88;
    }
    { // row 89
      double a64 = 0.0;
      a64 = fma(r1delt, ws[2007], a64);
      double a89 = 1.0;
      a89 = fma(-r1delt, ws[2173], a89);
      a89 = fma(-r1delt, ws[2175], a89);
      a89 = fma(-r1delt, ws[2177], a89);
      a89 = fma(-r1delt, ws[2179], a89);
      double a130 = 0.0;
      double a135 = 0.0;
      double a137 = 0.0;
      a137 = fma(-r1delt, ws[2174], a137);
      double a145 = 0.0;
      a145 = fma(r1delt, ws[2008], a145);
      a145 = fma(-r1delt, ws[2178], a145);
      double a146 = 0.0;
      a146 = fma(-r1delt, ws[2180], a146);
      double a147 = 0.0;
      a147 = fma(-r1delt, ws[2176], a147);
      double a148 = 0.0;
      a64 = a64 * CHEM_LDLU(vd + 64);
      lu[47] = a64;
      a130 = fma(-a64, CHEM_LDLU(lu + 1432), a130);
      a135 = fma(-a64, CHEM_LDLU(lu + 1433), a135);
      a145 = fma(-a64, CHEM_LDLU(lu + 1434), a145);
      a148 = fma(-a64, CHEM_LDLU(lu + 1435), a148);
      lu[1329] = a130;
      lu[1330] = a135;
      lu[1331] = a137;
      lu[1332] = a145;
      lu[1333] = a146;
      lu[1334] = a147;
      lu[1335] = a148;
      vd[89] = 1.0 / a89;
    }
    { // row 90
      double a90 = 1.0;
      a90 = fma(-r1delt, ws[1875], a90);
      a90 = fma(-r1delt, ws[1132], a90);
      double a134 = 0.0;
      a134 = fma(r1delt, ws[1867], a134);
      double a136 = 0.0;
      a136 = fma(r1delt, ws[1859], a136);
      double a143 = 0.0;
      a143 = fma(r1delt, ws[1851], a143);
      double a147 = 0.0;
      a147 = fma(r1delt, ws[1852], a147);
      a147 = fma(r1delt, ws[1860], a147);
      a147 = fma(r1delt, ws[1868], a147);
      double a148 = 0.0;
      a148 = fma(-r1delt, ws[1876], a148);
      lu[1324] = a134;
      lu[1325] = a136;
      lu[1326] = a143;
      lu[1327] = a147;
      lu[1328] = a148;
      vd[90] = 1.0 / a90;
    }
    { // row 91
      double a91 = 1.0;
      a91 = fma(-r1delt, ws[2209], a91);
      a91 = fma(0.2607 * r1delt, ws[2209], a91);
      double a99 = 0.0;
      a99 = fma(0.0491 * r1delt, ws[2211], a99);
      double a100 = 0.0;
      a100 = fma(0.064 * r1delt, ws[2213], a100);
      double a115 = 0.0;
      a115 = fma(0.0123 * r1delt, ws[2205], a115);
      double a116 = 0.0;
      a116 = fma(0.0139 * r1delt, ws[2207], a116);
      double a148 = 0.0;
      a148 = fma(0.0123 * r1delt, ws[2206], a148);
      a148 = fma(0.0139 * r1delt, ws[2208], a148);
      a148 = fma(-r1delt, ws[2210], a148);
      a148 = fma(0.2607 * r1delt, ws[2210], a148);
      a148 = fma(0.0491 * r1delt, ws[2212], a148);
      a148 = fma(0.064 * r1delt, ws[2214], a148);
      lu[1319] = a99;
      lu[1320] = a100;
      lu[1321] = a115;
      lu[1322] = a116;
      lu[1323] = a148;
      vd[91] = 1.0 / a91;
    }
    { // row 92
      double a34 = 0.0;
      a34 = fma(r1delt, ws[2027], a34);
      a34 = fma(r1delt, ws[2134], a34);
      double a92 = 1.0;
      a92 = fma(-r1delt, ws[2141], a92);
      a92 = fma(-r1delt, ws[2143], a92);
      double a137 = 0.0;
      a137 = fma(-r1delt, ws[2142], a137);
      double a142 = 0.0;
      a142 = fma(r1delt, ws[2133], a142);
      double a147 = 0.0;
      a147 = fma(-r1delt, ws[2144], a147);
      double a148 = 0.0;
      a148 = fma(r1delt, ws[2028], a148);
      a34 = a34 * CHEM_LDLU(vd + 34);
      lu[48] = a34;
      a142 = fma(-a34, CHEM_LDLU(lu + 1501), a142);
      a148 = fma(-a34, CHEM_LDLU(lu + 1502), a148);
      lu[1315] = a137;
      lu[1316] = a142;
      lu[1317] = a147;
      lu[1318] = a148;
      vd[92] = 1.0 / a92;
    }
    { // row 93
      double a75 = 0.0;
      a75 = fma(0.58 * r1delt, ws[2231], a75);
      a75 = fma(0.52 * r1delt, ws[2233], a75);
      a75 = fma(0.045 * r1delt, ws[2235], a75);
      a75 = fma(0.58 * r1delt, ws[2237], a75);
      double a93 = 1.0;
      a93 = fma(-r1delt, ws[2247], a93);
      a93 = fma(-r1delt, ws[2249], a93);
      a93 = fma(-r1delt, ws[2251], a93);
      a93 = fma(-r1delt, ws[1379], a93);
      a93 = fma(-r1delt, ws[2253], a93);
      double a135 = 0.0;
      a135 = fma(0.52 * r1delt, ws[2234], a135);
      a135 = fma(-r1delt, ws[2250], a135);
      double a142 = 0.0;
      a142 = fma(0.58 * r1delt, ws[2238], a142);
      a142 = fma(-r1delt, ws[2254], a142);
      double a145 = 0.0;
      a145 = fma(0.045 * r1delt, ws[2236], a145);
      a145 = fma(-r1delt, ws[2252], a145);
      double a148 = 0.0;
      a148 = fma(0.58 * r1delt, ws[2232], a148);
      a148 = fma(-r1delt, ws[2248], a148);
      a75 = a75 * CHEM_LDLU(vd + 75);
      lu[49] = a75;
      a135 = fma(-a75, CHEM_LDLU(lu + 1386), a135);
      a142 = fma(-a75, CHEM_LDLU(lu + 1387), a142);
      a145 = fma(-a75, CHEM_LDLU(lu + 1388), a145);
      a148 = fma(-a75, CHEM_LDLU(lu + 1389), a148);
      lu[1311] = a135;
      lu[1312] = a142;
      lu[1313] = a145;
      lu[1314] = a148;
      vd[93] = 1.0 / a93;
    }
    { // row 94
      double a37 = 0.0;
      a37 = fma(-r1delt, ws[2262], a37);
      double a94 = 1.0;
      a94 = fma(-r1delt, ws[2259], a94);
      a94 = fma(-r1delt, ws[2261], a94);
      a94 = fma(-r1delt, ws[2263], a94);
      a94 = fma(-r1delt, ws[2265], a94);
      a94 = fma(-r1delt, ws[2267], a94);
      a94 = fma(0.5 * r1delt, ws[2267], a94);
      double a108 = 0.0;
      a108 = fma(-r1delt, ws[2264], a108);
      double a110 = 0.0;
      double a135 = 0.0;
      a135 = fma(-r1delt, ws[2260], a135);
      double a142 = 0.0;
      a142 = fma(-r1delt, ws[2268], a142);
      a142 = fma(0.5 * r1delt, ws[2268], a142);
      double a148 = 0.0;
      a148 = fma(-r1delt, ws[2266], a148);
      a37 = a37 * CHEM_LDLU(vd + 37);
      lu[50] = a37;
      a94 = fma(-a37, CHEM_LDLU(lu + 1495), a94);
      a110 = fma(-a37, CHEM_LDLU(lu + 1496), a110);
      lu[1306] = a108;
      lu[1307] = a110;
      lu[1308] = a135;
      lu[1309] = a142;
      lu[1310] = a148;
      vd[94] = 1.0 / a94;
    }
    { // row 95
      double a37 = 0.0;
      a37 = fma(r1delt, ws[2262], a37);
      double a94 = 0.0;
      a94 = fma(0.5 * r1delt, ws[2259], a94);
      a94 = fma(r1delt, ws[2261], a94);
      a94 = fma(r1delt, ws[2263], a94);
      a94 = fma(0.5 * r1delt, ws[2265], a94);
      a94 = fma(0.5 * r1delt, ws[2267], a94);
      double a95 = 1.0;
      double a108 = 0.0;
      a108 = fma(r1delt, ws[2264], a108);
      double a110 = 0.0;
      double a135 = 0.0;
      a135 = fma(0.5 * r1delt, ws[2260], a135);
      double a142 = 0.0;
      a142 = fma(0.5 * r1delt, ws[2268], a142);
      double a148 = 0.0;
      a148 = fma(0.5 * r1delt, ws[2266], a148);
      a37 = a37 * CHEM_LDLU(vd + 37);
      lu[51] = a37;
      a94 = fma(-a37, CHEM_LDLU(lu + 1495), a94);
      a110 = fma(-a37, CHEM_LDLU(lu + 1496), a110);
      a94 = a94 * CHEM_LDLU(vd + 94);
      lu[52] = a94;
      a108 = fma(-a94, CHEM_LDLU(lu + 1306), a108);
      a110 = fma(-a94, CHEM_LDLU(lu + 1307), a110);
      a135 = fma(-a94, CHEM_LDLU(lu + 1308), a135);
      a142 = fma(-a94, CHEM_LDLU(lu + 1309), a142);
      a148 = fma(-a94, CHEM_LDLU(lu + 1310), a148);
      lu[1301] = a108;
      lu[1302] = a110;
      lu[1303] = a135;
      lu[1304] = a142;
      lu[1305] = a148;
      vd[95] = 1.0 / a95;
    }
    { // row 96
      double a14 = 0.0;
      a14 = fma(0.081 * r1delt, ws[2163], a14);
      double a67 = 0.0;
      a67 = fma(0.392 * r1delt, ws[2149], a67);
      double a78 = 0.0;
      a78 = fma(0.06 * r1delt, ws[2145], a78);
      double a80 = 0.0;
      a80 = fma(0.191 * r1delt, ws[2159], a80);
      double a92 = 0.0;
      a92 = fma(0.047 * r1delt, ws[2141], a92);
      double a96 = 1.0;
      double a137 = 0.0;
      a137 = fma(0.047 * r1delt, ws[2142], a137);
      a137 = fma(0.06 * r1delt, ws[2146], a137);
      a137 = fma(0.392 * r1delt, ws[2150], a137);
      a137 = fma(0.191 * r1delt, ws[2160], a137);
      double a142 = 0.0;
      double a147 = 0.0;
      double a148 = 0.0;
      a148 = fma(0.081 * r1delt, ws[2164], a148);
      a14 = a14 * CHEM_LDLU(vd + 14);
      lu[53] = a14;
      a148 = fma(-a14, CHEM_LDLU(lu + 1532), a148);
      a67 = a67 * CHEM_LDLU(vd + 67);
      lu[54] = a67;
      a137 = fma(-a67, CHEM_LDLU(lu + 1420), a137);
      a147 = fma(-a67, CHEM_LDLU(lu + 1421), a147);
      a148 = fma(-a67, CHEM_LDLU(lu + 1422), a148);
      a78 = a78 * CHEM_LDLU(vd + 78);
      lu[55] = a78;
      a137 = fma(-a78, CHEM_LDLU(lu + 1373), a137);
      a142 = fma(-a78, CHEM_LDLU(lu + 1374), a142);
      a147 = fma(-a78, CHEM_LDLU(lu + 1375), a147);
      a148 = fma(-a78, CHEM_LDLU(lu + 1376), a148);
      a80 = a80 * CHEM_LDLU(vd + 80);
      lu[56] = a80;
      a137 = fma(-a80, CHEM_LDLU(lu + 1364), a137);
      a142 = fma(-a80, CHEM_LDLU(lu + 1365), a142);
      a147 = fma(-a80, CHEM_LDLU(lu + 1366), a147);
      a148 = fma(-a80, CHEM_LDLU(lu + 1367), a148);
      a92 = a92 * CHEM_LDLU(vd + 92);
      lu[57] = a92;
      a137 = fma(-a92, CHEM_LDLU(lu + 1315), a137);
      a142 = fma(-a92, CHEM_LDLU(lu + 1316), a142);
      a147 = fma(-a92, CHEM_LDLU(lu + 1317), a147);
      a148 = fma(-a92, CHEM_LDLU(lu + 1318), a148);
      lu[1297] = a137;
      lu[1298] = a142;
      lu[1299] = a147;
      lu[1300] = a148;
      vd[96] = 1.0 / a96;
    }
    { // row 97
      double a12 = 0.0;
      a12 = fma(0.352 * r1delt, ws[2017], a12);
      double a97 = 1.0;
      a97 = fma(-r1delt, ws[2019], a97);
      a97 = fma(-r1delt, ws[2021], a97);
      a97 = fma(-r1delt, ws[2023], a97);
      a97 = fma(-r1delt, ws[2025], a97);
      double a137 = 0.0;
      a137 = fma(-r1delt, ws[2020], a137);
      double a139 = 0.0;
      a139 = fma(-r1delt, ws[2022], a139);
      double a146 = 0.0;
      a146 = fma(-r1delt, ws[2026], a146);
      double a147 = 0.0;
      a147 = fma(-r1delt, ws[2024], a147);
      double a148 = 0.0;
      a148 = fma(0.352 * r1delt, ws[2018], a148);
      a12 = a12 * CHEM_LDLU(vd + 12);
      lu[58] = a12;
      a148 = fma(-a12, CHEM_LDLU(lu + 1534), a148);
      lu[1292] = a137;
      lu[1293] = a139;
      lu[1294] = a146;
      lu[1295] = a147;
      lu[1296] = a148;
      vd[97] = 1.0 / a97;
    }
    { // row 98
      double a52 = 0.0;
      a52 = fma(0.029 * r1delt, ws[1985], a52);
      double a98 = 1.0;
      a98 = fma(-r1delt, ws[1955], a98);
      a98 = fma(-r1delt, ws[1957], a98);
      a98 = fma(-r1delt, ws[1959], a98);
      a98 = fma(-r1delt, ws[1961], a98);
      a98 = fma(-r1delt, ws[2118], a98);
      double a107 = 0.0;
      double a130 = 0.0;
      a130 = fma(-r1delt, ws[1956], a130);
      double a135 = 0.0;
      a135 = fma(-r1delt, ws[1960], a135);
      double a142 = 0.0;
      a142 = fma(-r1delt, ws[2117], a142);
      double a145 = 0.0;
      a145 = fma(-r1delt, ws[1962], a145);
      double a147 = 0.0;
      double a148 = 0.0;
      a148 = fma(-r1delt, ws[1958], a148);
      a148 = fma(0.029 * r1delt, ws[1986], a148);
      a52 = a52 * CHEM_LDLU(vd + 52);
      lu[59] = a52;
      a107 = fma(-a52, CHEM_LDLU(lu + 1468), a107);
      a147 = fma(-a52, CHEM_LDLU(lu + 1469), a147);
      a148 = fma(-a52, CHEM_LDLU(lu + 1470), a148);
      lu[1285] = a107;
      lu[1286] = a130;
      lu[1287] = a135;
      lu[1288] = a142;
      lu[1289] = a145;
      lu[1290] = a147;
      lu[1291] = a148;
      vd[98] = 1.0 / a98;
    }
    { // row 99
      double a86 = 0.0;
      a86 = fma(0.0019 * r1delt, ws[2195], a86);
      double a87 = 0.0;
      double a88 = 0.0;
      double a91 = 0.0;
      a91 = fma(0.0702 * r1delt, ws[2209], a91);
      double a99 = 1.0;
      a99 = fma(-r1delt, ws[2211], a99);
      a99 = fma(0.2577 * r1delt, ws[2211], a99);
      double a100 = 0.0;
      a100 = fma(0.0385 * r1delt, ws[2213], a100);
      double a115 = 0.0;
      a115 = fma(0.1239 * r1delt, ws[2205], a115);
      double a116 = 0.0;
      a116 = fma(0.1027 * r1delt, ws[2207], a116);
      double a148 = 0.0;
      a148 = fma(0.0019 * r1delt, ws[2196], a148);
      a148 = fma(0.1239 * r1delt, ws[2206], a148);
      a148 = fma(0.1027 * r1delt, ws[2208], a148);
      a148 = fma(0.0702 * r1delt, ws[2210], a148);
      a148 = fma(-r1delt, ws[2212], a148);
      a148 = fma(0.2577 * r1delt, ws[2212], a148);
      a148 = fma(0.0385 * r1delt, ws[2214], a148);
      a86 = a86 * CHEM_LDLU(vd + 86);
      lu[60] = a86;
      a87 = fma(-a86, CHEM_LDLU(lu + 1339), a87);
      a88 = fma(-a86, CHEM_LDLU(lu + 1340), a88);
      a148 = fma(-a86, CHEM_LDLU(lu + 1341), a148);
      a87 = a87 * CHEM_LDLU(vd + 87);
      lu[61] = a87;
      a88 = fma(-a87, CHEM_LDLU(lu + 1337), a88);
      a148 = fma(-a87, CHEM_LDLU(lu + 1338), a148);
      a88 = a88 * CHEM_LDLU(vd + 88);
      lu[62] = a88;
      a148 = fma(-a88, CHEM_LDLU(lu + 1336), a148);
      a91 = a91 * CHEM_LDLU(vd + 91);
      lu[63] = a91;
      a99 = fma(-a91, CHEM_LDLU(lu + 1319), a99);
      a100 = fma(-a91, CHEM_LDLU(lu + 1320), a100);
      a115 = fma(-a91, CHEM_LDLU(lu + 1321), a115);
      a116 = fma(-a91, CHEM_LDLU(lu + 1322), a116);
      a148 = fma(-a91, CHEM_LDLU(lu + 1323), a148);
      lu[1281] = a100;
      lu[1282] = a115;
      lu[1283] = a116;
      lu[1284] = a148;
      vd[99] = 1.0 / a99;
    }
    { // row 100
      double a86 = 0.0;
      a86 = fma(0.0023 * r1delt, ws[2195], a86);
      double a87 = 0.0;
      double a88 = 0.0;
      double a91 = 0.0;
      a91 = fma(0.1116 * r1delt, ws[2209], a91);
      double a99 = 0.0;
      a99 = fma(0.0739 * r1delt, ws[2211], a99);
      double a100 = 1.0;
      a100 = fma(-r1delt, ws[2213], a100);
      a100 = fma(0.2667 * r1delt, ws[2213], a100);
      double a115 = 0.0;
      a115 = fma(0.1831 * r1delt, ws[2205], a115);
      double a116 = 0.0;
      a116 = fma(0.2045 * r1delt, ws[2207], a116);
      double a148 = 0.0;
      a148 = fma(0.0023 * r1delt, ws[2196], a148);
      a148 = fma(0.1831 * r1delt, ws[2206], a148);
      a148 = fma(0.2045 * r1delt, ws[2208], a148);
      a148 = fma(0.1116 * r1delt, ws[2210], a148);
      a148 = fma(0.0739 * r1delt, ws[2212], a148);
      a148 = fma(-r1delt, ws[2214], a148);
      a148 = fma(0.2667 * r1delt, ws[2214], a148);
      a86 = a86 * CHEM_LDLU(vd + 86);
      lu[64] = a86;
      a87 = fma(-a86, CHEM_LDLU(lu + 1339), a87);
      a88 = fma(-a86, CHEM_LDLU(lu + 1340), a88);
      a148 = fma(-a86, CHEM_LDLU(lu + 1341), a148);
      a87 = a87 * CHEM_LDLU(vd + 87);
      lu[65] = a87;
      a88 = fma(-a87, CHEM_LDLU(lu + 1337), a88);
      a148 = fma(-a87, CHEM_LDLU(lu + 1338), a148);
      a88 = a88 * CHEM_LDLU(vd + 88);
      lu[66] = a88;
      a148 = fma(-a88, CHEM_LDLU(lu + 1336), a148);
      a91 = a91 * CHEM_LDLU(vd + 91);
      lu[67] = a91;
      a99 = fma(-a91, CHEM_LDLU(lu + 1319), a99);
      a100 = fma(-a91, CHEM_LDLU(lu + 1320), a100);
      a115 = fma(-a91, CHEM_LDLU(lu + 1321), a115);
      a116 = fma(-a91, CHEM_LDLU(lu + 1322), a116);
      a148 = fma(-a91, CHEM_LDLU(lu + 1323), a148);
      a99 = a99 * CHEM_LDLU(vd + 99);
      lu[68] = a99;
      a100 = fma(-a99, CHEM_LDLU(lu + 1281), a100);
      a115 = fma(-a99, CHEM_LDLU(lu + 1282), a115);
      a116 = fma(-a99, CHEM_LDLU(lu + 1283), a116);
      a148 = fma(-a99, CHEM_LDLU(lu + 1284), a148);
      lu[1278] = a115;
      lu[1279] = a116;
      lu[1280] = a148;
      vd[100] = 1.0 / a100;
    }
}
}  // namespace mech_cb6r5_ae7_aq
