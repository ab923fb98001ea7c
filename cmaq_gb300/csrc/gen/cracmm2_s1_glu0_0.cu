// Generated by cmaq_gb300.mechgen.generate from CCTM/src/MECHS/cracmm2/RXNS_DATA_MODULE.F90
// and RXNS_FUNC_MODULE.F90 (sha256/16 61a0c9d4d7262bbb).  Do not edit.
#include "cracmm2_mech.cuh"
#include <math.h>
namespace mech_cracmm2 {
__device__ __noinline__ void gear_pdecomp_s1_0_0(double* __restrict__ ws, double r1delt)
{
    double* __restrict__ lu = ws + 3484;
    double* __restrict__ vd = ws + 6769;
    { // row 0
      double a0 = 1.0;
      double a33 = 0.0;
      a33 = fma(r1delt, ws[1751], a33);
      lu[3095] = a33;
      vd[0] = 1.0 / a0;
    }
    { // row 1
      double a1 = 1.0;
      double a52 = 0.0;
      a52 = fma(r1delt, ws[1753], a52);
      lu[3094] = a52;
      vd[1] = 1.0 / a1;
    }
    { // row 2
      double a2 = 1.0;
      double a69 = 0.0;
      a69 = fma(r1delt, ws[1754], a69);
      lu[3093] = a69;
      vd[2] = 1.0 / a2;
    }
    { // row 3
      double a3 = 1.0;
      a3 = fma(-r1delt, ws[1846], a3);
      vd[3] = 1.0 / a3;
    }
    { // row 4
      double a4 = 1.0;
      a4 = fma(-r1delt, ws[1847], a4);
      vd[4] = 1.0 / a4;
    }
    { // row 5
      double a5 = 1.0;
      a5 = fma(-r1delt, ws[2439], a5);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[2440], a188);
      lu[3092] = a188;
      vd[5] = 1.0 / a5;
    }
    { // row 6
      double a5 = 0.0;
      a5 = fma(r1delt, ws[2439], a5);
      double a6 = 1.0;
      double a188 = 0.0;
      a188 = fma(r1delt, ws[2440], a188);
      a5 = a5 * CHEM_LDLU(vd + 5);
      lu[1] = a5;
      a188 = fma(-a5, CHEM_LDLU(lu + 3092), a188);
      lu[3091] = a188;
      vd[6] = 1.0 / a6;
    }
    { // row 7
      double a5 = 0.0;
      a5 = fma(r1delt, ws[2439], a5);
      double a7 = 1.0;
      double a188 = 0.0;
      a188 = fma(r1delt, ws[2440], a188);
      a5 = a5 * CHEM_LDLU(vd + 5);
      lu[2] = a5;
      a188 = fma(-a5, CHEM_LDLU(lu + 3092), a188);
      lu[3090] = a188;
      vd[7] = 1.0 / a7;
    }
    { // row 8
      double a8 = 1.0;
      a8 = fma(-r1delt, ws[2455], a8);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[2456], a188);
      lu[3089] = a188;
      vd[8] = 1.0 / a8;
    }
    { // row 9
      double a9 = 1.0;
      a9 = fma(-r1delt, ws[2459], a9);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[2460], a188);
      lu[3088] = a188;
      vd[9] = 1.0 / a9;
    }
    { // row 10
      double a10 = 1.0;
      a10 = fma(-r1delt, ws[2461], a10);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[2462], a188);
      lu[3087] = a188;
      vd[10] = 1.0 / a10;
    }
    { // row 11
      double a11 = 1.0;
      a11 = fma(-r1delt, ws[2463], a11);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[2464], a188);
      lu[3086] = a188;
      vd[11] = 1.0 / a11;
    }
    { // row 12
      double a12 = 1.0;
      a12 = fma(-r1delt, ws[3055], a12);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[3056], a188);
      lu[3085] = a188;
      vd[12] = 1.0 / a12;
    }
    { // row 13
      double a13 = 1.0;
      a13 = fma(-r1delt, ws[3057], a13);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[3058], a188);
      lu[3084] = a188;
      vd[13] = 1.0 / a13;
    }
    { // row 14
      double a14 = 1.0;
      a14 = fma(-r1delt, ws[3093], a14);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[3094], a188);
      lu[3083] = a188;
      vd[14] = 1.0 / a14;
    }
    { // row 15
      double a15 = 1.0;
      double a164 = 0.0;
      a164 = fma(r1delt, ws[1744], a164);
      double a168 = 0.0;
      a168 = fma(r1delt, ws[1743], a168);
      lu[3081] = a164;
      lu[3082] = a168;
      vd[15] = 1.0 / a15;
    }
    { // row 16
      double a16 = 1.0;
      a16 = fma(-r1delt, ws[3114], a16);
      double a33 = 0.0;
      a33 = fma(-r1delt, ws[3113], a33);
      lu[3080] = a33;
      vd[16] = 1.0 / a16;
    }
    { // row 17
      double a16 = 0.0;
      a16 = fma(r1delt, ws[3114], a16);
      double a17 = 1.0;
      double a33 = 0.0;
      a33 = fma(r1delt, ws[3113], a33);
      a16 = a16 * CHEM_LDLU(vd + 16);
      lu[3] = a16;
      a33 = fma(-a16, CHEM_LDLU(lu + 3080), a33);
      lu[3079] = a33;
      vd[17] = 1.0 / a17;
    }
    { // row 18
      double a18 = 1.0;
      a18 = fma(-r1delt, ws[1369], a18);
      a18 = fma(-r1delt, ws[1370], a18);
      a18 = fma(-r1delt, ws[1371], a18);
      double a162 = 0.0;
      a162 = fma(r1delt, ws[1324], a162);
      lu[3078] = a162;
      vd[18] = 1.0 / a18;
    }
    { // row 19
      double a19 = 1.0;
      a19 = fma(-r1delt, ws[3115], a19);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[3116], a188);
      lu[3077] = a188;
      vd[19] = 1.0 / a19;
    }
    { // row 20
      double a20 = 1.0;
      a20 = fma(-r1delt, ws[3117], a20);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[3118], a188);
      lu[3076] = a188;
      vd[20] = 1.0 / a20;
    }
    { // row 21
      double a21 = 1.0;
      a21 = fma(-r1delt, ws[3119], a21);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[3120], a188);
      lu[3075] = a188;
      vd[21] = 1.0 / a21;
    }
    { // row 22
      double a22 = 1.0;
      a22 = fma(-r1delt, ws[3121], a22);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[3122], a188);
      lu[3074] = a188;
      vd[22] = 1.0 / a22;
    }
    { // row 23
      double a23 = 1.0;
      a23 = fma(-r1delt, ws[3123], a23);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[3124], a188);
      lu[3073] = a188;
      vd[23] = 1.0 / a23;
    }
    { // row 24
      double a24 = 1.0;
      a24 = fma(-r1delt, ws[3125], a24);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[3126], a188);
      lu[3072] = a188;
      vd[24] = 1.0 / a24;
    }
    { // row 25
      double a25 = 1.0;
      a25 = fma(-r1delt, ws[3127], a25);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[3128], a188);
      lu[3071] = a188;
      vd[25] = 1.0 / a25;
    }
    { // row 26
      double a26 = 1.0;
      a26 = fma(-r1delt, ws[3213], a26);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[3214], a188);
      lu[3070] = a188;
      vd[26] = 1.0 / a26;
    }
    { // row 27
      double a27 = 1.0;
      a27 = fma(-r1delt, ws[3225], a27);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[3226], a188);
      lu[3069] = a188;
      vd[27] = 1.0 / a27;
    }
    { // row 28
      double a28 = 1.0;
      a28 = fma(-r1delt, ws[3237], a28);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[3238], a188);
      lu[3068] = a188;
      vd[28] = 1.0 / a28;
    }
    { // row 29
      double a29 = 1.0;
      a29 = fma(-r1delt, ws[3281], a29);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[3282], a188);
      lu[3067] = a188;
      vd[29] = 1.0 / a29;
    }
    { // row 30
      double a3 = 0.0;
      a3 = fma(r1delt, ws[1846], a3);
      double a4 = 0.0;
      a4 = fma(r1delt, ws[1847], a4);
      double a30 = 1.0;
      a3 = a3 * CHEM_LDLU(vd + 3);
      lu[4] = a3;
      a4 = a4 * CHEM_LDLU(vd + 4);
      lu[5] = a4;
      vd[30] = 1.0 / a30;
    }
    { // row 31
      double a31 = 1.0;
      a31 = fma(-r1delt, ws[3283], a31);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[3284], a188);
      lu[3066] = a188;
      vd[31] = 1.0 / a31;
    }
    { // row 32
      double a32 = 1.0;
      a32 = fma(-r1delt, ws[1393], a32);
      a32 = fma(-r1delt, ws[1394], a32);
      a32 = fma(-r1delt, ws[1745], a32);
      double a185 = 0.0;
      a185 = fma(r1delt, ws[2434], a185);
      double a186 = 0.0;
      a186 = fma(r1delt, ws[2433], a186);
      lu[3064] = a185;
      lu[3065] = a186;
      vd[32] = 1.0 / a32;
    }
    { // row 33
      double a16 = 0.0;
      a16 = fma(-r1delt, ws[3114], a16);
      double a33 = 1.0;
      a33 = fma(-r1delt, ws[1751], a33);
      a33 = fma(-r1delt, ws[3113], a33);
      double a43 = 0.0;
      a43 = fma(r1delt, ws[1750], a43);
      a16 = a16 * CHEM_LDLU(vd + 16);
      lu[6] = a16;
      a33 = fma(-a16, CHEM_LDLU(lu + 3080), a33);
      lu[3063] = a43;
      vd[33] = 1.0 / a33;
    }
    { // row 34
      double a34 = 1.0;
      a34 = fma(-r1delt, ws[1359], a34);
      a34 = fma(-r1delt, ws[1360], a34);
      a34 = fma(-r1delt, ws[2559], a34);
      a34 = fma(-r1delt, ws[1500], a34);
      double a181 = 0.0;
      a181 = fma(r1delt, ws[2633], a181);
      double a185 = 0.0;
      a185 = fma(r1delt, ws[2634], a185);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[2560], a188);
      lu[3060] = a181;
      lu[3061] = a185;
      lu[3062] = a188;
      vd[34] = 1.0 / a34;
    }
    { // row 35
      double a35 = 1.0;
      a35 = fma(-r1delt, ws[2447], a35);
      double a86 = 0.0;
      a86 = fma(0.006 * r1delt, ws[2573], a86);
      double a162 = 0.0;
      a162 = fma(0.006 * r1delt, ws[2574], a162);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[2448], a188);
      lu[3057] = a86;
      lu[3058] = a162;
      lu[3059] = a188;
      vd[35] = 1.0 / a35;
    }
    { // row 36
      double a36 = 1.0;
      a36 = fma(-r1delt, ws[2453], a36);
      a36 = fma(-r1delt, ws[2575], a36);
      a36 = fma(-r1delt, ws[2603], a36);
      double a162 = 0.0;
      a162 = fma(-r1delt, ws[2576], a162);
      double a186 = 0.0;
      a186 = fma(-r1delt, ws[2604], a186);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[2454], a188);
      lu[3054] = a162;
      lu[3055] = a186;
      lu[3056] = a188;
      vd[36] = 1.0 / a36;
    }
    { // row 37
      double a37 = 1.0;
      a37 = fma(-r1delt, ws[1329], a37);
      a37 = fma(-r1delt, ws[2413], a37);
      double a182 = 0.0;
      a182 = fma(r1delt, ws[2405], a182);
      double a185 = 0.0;
      a185 = fma(0.5 * r1delt, ws[1746], a185);
      double a188 = 0.0;
      a188 = fma(r1delt, ws[2406], a188);
      a188 = fma(-r1delt, ws[2414], a188);
      lu[3051] = a182;
      lu[3052] = a185;
      lu[3053] = a188;
      vd[37] = 1.0 / a37;
    }
    { // row 38
      double a38 = 1.0;
      a38 = fma(-r1delt, ws[2457], a38);
      double a86 = 0.0;
      a86 = fma(0.032 * r1delt, ws[2573], a86);
      double a162 = 0.0;
      a162 = fma(0.032 * r1delt, ws[2574], a162);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[2458], a188);
      lu[3048] = a86;
      lu[3049] = a162;
      lu[3050] = a188;
      vd[38] = 1.0 / a38;
    }
    { // row 39
      double a38 = 0.0;
      a38 = fma(0.53 * r1delt, ws[2457], a38);
      double a39 = 1.0;
      a39 = fma(-r1delt, ws[2529], a39);
      a39 = fma(-r1delt, ws[2625], a39);
      double a86 = 0.0;
      double a162 = 0.0;
      double a186 = 0.0;
      a186 = fma(-r1delt, ws[2626], a186);
      double a188 = 0.0;
      a188 = fma(0.53 * r1delt, ws[2458], a188);
      a188 = fma(-r1delt, ws[2530], a188);
      a38 = a38 * CHEM_LDLU(vd + 38);
      lu[7] = a38;
      a86 = fma(-a38, CHEM_LDLU(lu + 3048), a86);
      a162 = fma(-a38, CHEM_LDLU(lu + 3049), a162);
      a188 = fma(-a38, CHEM_LDLU(lu + 3050), a188);
      lu[3044] = a86;
      lu[3045] = a162;
      lu[3046] = a186;
      lu[3047] = a188;
      vd[39] = 1.0 / a39;
    }
    { // row 40
      double a40 = 1.0;
      a40 = fma(-r1delt, ws[1331], a40);
      a40 = fma(-r1delt, ws[1396], a40);
      a40 = fma(-r1delt, ws[2437], a40);
      double a185 = 0.0;
      a185 = fma(r1delt, ws[2435], a185);
      double a187 = 0.0;
      a187 = fma(r1delt, ws[2436], a187);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[2438], a188);
      lu[3041] = a185;
      lu[3042] = a187;
      lu[3043] = a188;
      vd[40] = 1.0 / a40;
    }
    { // row 41
      double a41 = 1.0;
      a41 = fma(-r1delt, ws[2465], a41);
      a41 = fma(-r1delt, ws[2467], a41);
      a41 = fma(-r1delt, ws[2469], a41);
      double a162 = 0.0;
      a162 = fma(-r1delt, ws[2466], a162);
      double a186 = 0.0;
      a186 = fma(-r1delt, ws[2468], a186);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[2470], a188);
      lu[3038] = a162;
      lu[3039] = a186;
      lu[3040] = a188;
      vd[41] = 1.0 / a41;
    }
    { // row 42
      double a42 = 1.0;
      a42 = fma(-r1delt, ws[2475], a42);
      a42 = fma(-r1delt, ws[2477], a42);
      double a134 = 0.0;
      a134 = fma(r1delt, ws[2471], a134);
      double a187 = 0.0;
      a187 = fma(r1delt, ws[2472], a187);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[2476], a188);
      a188 = fma(-r1delt, ws[2478], a188);
      lu[3035] = a134;
      lu[3036] = a187;
      lu[3037] = a188;
      vd[42] = 1.0 / a42;
    }
    { // row 43
      double a42 = 0.0;
      a42 = fma(0.44 * r1delt, ws[2477], a42);
      double a43 = 1.0;
      a43 = fma(-r1delt, ws[3053], a43);
      a43 = fma(-r1delt, ws[1750], a43);
      double a87 = 0.0;
      a87 = fma(0.17 * r1delt, ws[2483], a87);
      double a134 = 0.0;
      double a187 = 0.0;
      double a188 = 0.0;
      a188 = fma(0.44 * r1delt, ws[2478], a188);
      a188 = fma(0.17 * r1delt, ws[2484], a188);
      a188 = fma(-r1delt, ws[3054], a188);
      a42 = a42 * CHEM_LDLU(vd + 42);
      lu[8] = a42;
      a134 = fma(-a42, CHEM_LDLU(lu + 3035), a134);
      a187 = fma(-a42, CHEM_LDLU(lu + 3036), a187);
      a188 = fma(-a42, CHEM_LDLU(lu + 3037), a188);
      lu[3031] = a87;
      lu[3032] = a134;
      lu[3033] = a187;
      lu[3034] = a188;
      vd[43] = 1.0 / a43;
    }
    { // row 44
      double a44 = 1.0;
      a44 = fma(-r1delt, ws[2489], a44);
      a44 = fma(-r1delt, ws[2577], a44);
      a44 = fma(-r1delt, ws[2605], a44);
      double a162 = 0.0;
      a162 = fma(-r1delt, ws[2578], a162);
      double a186 = 0.0;
      a186 = fma(-r1delt, ws[2606], a186);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[2490], a188);
      lu[3028] = a162;
      lu[3029] = a186;
      lu[3030] = a188;
      vd[44] = 1.0 / a44;
    }
    { // row 45
      double a45 = 1.0;
      a45 = fma(-r1delt, ws[2491], a45);
      a45 = fma(-r1delt, ws[2579], a45);
      a45 = fma(-r1delt, ws[2607], a45);
      double a162 = 0.0;
      a162 = fma(-r1delt, ws[2580], a162);
      double a186 = 0.0;
      a186 = fma(-r1delt, ws[2608], a186);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[2492], a188);
      lu[3025] = a162;
      lu[3026] = a186;
      lu[3027] = a188;
      vd[45] = 1.0 / a45;
    }
    { // row 46
      double a46 = 1.0;
      a46 = fma(-r1delt, ws[2537], a46);
      double a176 = 0.0;
      a176 = fma(0.25 * r1delt, ws[2801], a176);
      double a184 = 0.0;
      a184 = fma(0.25 * r1delt, ws[2802], a184);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[2538], a188);
      lu[3022] = a176;
      lu[3023] = a184;
      lu[3024] = a188;
      vd[46] = 1.0 / a46;
    }
    { // row 47
      double a47 = 1.0;
      a47 = fma(-r1delt, ws[2541], a47);
      double a94 = 0.0;
      a94 = fma(0.25 * r1delt, ws[2807], a94);
      double a184 = 0.0;
      a184 = fma(0.25 * r1delt, ws[2808], a184);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[2542], a188);
      lu[3019] = a94;
      lu[3020] = a184;
      lu[3021] = a188;
      vd[47] = 1.0 / a47;
    }
    { // row 48
      double a48 = 1.0;
      a48 = fma(-r1delt, ws[2561], a48);
      a48 = fma(-r1delt, ws[1502], a48);
      double a150 = 0.0;
      a150 = fma(r1delt, ws[2635], a150);
      double a185 = 0.0;
      a185 = fma(r1delt, ws[2636], a185);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[2562], a188);
      lu[3016] = a150;
      lu[3017] = a185;
      lu[3018] = a188;
      vd[48] = 1.0 / a48;
    }
    { // row 49
      double a49 = 1.0;
      a49 = fma(-r1delt, ws[3065], a49);
      a49 = fma(-r1delt, ws[3077], a49);
      a49 = fma(-r1delt, ws[3079], a49);
      double a162 = 0.0;
      a162 = fma(-r1delt, ws[3078], a162);
      double a186 = 0.0;
      a186 = fma(-r1delt, ws[3080], a186);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[3066], a188);
      lu[3013] = a162;
      lu[3014] = a186;
      lu[3015] = a188;
      vd[49] = 1.0 / a49;
    }
    { // row 50
      double a50 = 1.0;
      a50 = fma(-r1delt, ws[3095], a50);
      a50 = fma(-r1delt, ws[3103], a50);
      a50 = fma(-r1delt, ws[3105], a50);
      double a162 = 0.0;
      a162 = fma(-r1delt, ws[3104], a162);
      double a186 = 0.0;
      a186 = fma(-r1delt, ws[3096], a186);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[3106], a188);
      lu[3010] = a162;
      lu[3011] = a186;
      lu[3012] = a188;
      vd[50] = 1.0 / a50;
    }
    { // row 51
      double a41 = 0.0;
      a41 = fma(0.555 * r1delt, ws[2467], a41);
      double a51 = 1.0;
      a51 = fma(-r1delt, ws[2479], a51);
      a51 = fma(-r1delt, ws[2481], a51);
      double a162 = 0.0;
      double a182 = 0.0;
      a182 = fma(-r1delt, ws[2482], a182);
      double a186 = 0.0;
      a186 = fma(0.555 * r1delt, ws[2468], a186);
      double a187 = 0.0;
      a187 = fma(-r1delt, ws[2480], a187);
      double a188 = 0.0;
      a41 = a41 * CHEM_LDLU(vd + 41);
      lu[9] = a41;
      a162 = fma(-a41, CHEM_LDLU(lu + 3038), a162);
      a186 = fma(-a41, CHEM_LDLU(lu + 3039), a186);
      a188 = fma(-a41, CHEM_LDLU(lu + 3040), a188);
      lu[3005] = a162;
      lu[3006] = a182;
      lu[3007] = a186;
      lu[3008] = a187;
      lu[3009] = a188;
      vd[51] = 1.0 / a51;
    }
    { // row 52
      double a42 = 0.0;
      a42 = fma(0.14 * r1delt, ws[2477], a42);
      double a51 = 0.0;
      a51 = fma(0.02 * r1delt, ws[2479], a51);
      double a52 = 1.0;
      a52 = fma(-r1delt, ws[2487], a52);
      a52 = fma(-r1delt, ws[1753], a52);
      double a134 = 0.0;
      double a162 = 0.0;
      double a182 = 0.0;
      double a186 = 0.0;
      double a187 = 0.0;
      a187 = fma(0.02 * r1delt, ws[2480], a187);
      double a188 = 0.0;
      a188 = fma(0.14 * r1delt, ws[2478], a188);
      a188 = fma(-r1delt, ws[2488], a188);
      a42 = a42 * CHEM_LDLU(vd + 42);
      lu[10] = a42;
      a134 = fma(-a42, CHEM_LDLU(lu + 3035), a134);
      a187 = fma(-a42, CHEM_LDLU(lu + 3036), a187);
      a188 = fma(-a42, CHEM_LDLU(lu + 3037), a188);
      a51 = a51 * CHEM_LDLU(vd + 51);
      lu[11] = a51;
      a162 = fma(-a51, CHEM_LDLU(lu + 3005), a162);
      a182 = fma(-a51, CHEM_LDLU(lu + 3006), a182);
      a186 = fma(-a51, CHEM_LDLU(lu + 3007), a186);
      a187 = fma(-a51, CHEM_LDLU(lu + 3008), a187);
      a188 = fma(-a51, CHEM_LDLU(lu + 3009), a188);
      lu[2999] = a134;
      lu[3000] = a162;
      lu[3001] = a182;
      lu[3002] = a186;
      lu[3003] = a187;
      lu[3004] = a188;
      vd[52] = 1.0 / a52;
    }
    { // row 53
      double a53 = 1.0;
      a53 = fma(-r1delt, ws[1362], a53);
      a53 = fma(-r1delt, ws[2569], a53);
      double a137 = 0.0;
      a137 = fma(0.33 * r1delt, ws[2567], a137);
      a137 = fma(0.33 * r1delt, ws[2583], a137);
      a137 = fma(0.33 * r1delt, ws[2609], a137);
      double a162 = 0.0;
      a162 = fma(0.33 * r1delt, ws[2584], a162);
      double a186 = 0.0;
      a186 = fma(0.33 * r1delt, ws[2610], a186);
      double a188 = 0.0;
      a188 = fma(0.33 * r1delt, ws[2568], a188);
      a188 = fma(-r1delt, ws[2570], a188);
      lu[2995] = a137;
      lu[2996] = a162;
      lu[2997] = a186;
      lu[2998] = a188;
      vd[53] = 1.0 / a53;
    }
    { // row 54
      double a54 = 1.0;
      a54 = fma(-r1delt, ws[1498], a54);
      a54 = fma(-r1delt, ws[2679], a54);
      a54 = fma(-r1delt, ws[2763], a54);
      double a143 = 0.0;
      a143 = fma(0.83 * r1delt, ws[2495], a143);
      double a182 = 0.0;
      a182 = fma(-r1delt, ws[2680], a182);
      double a187 = 0.0;
      a187 = fma(-r1delt, ws[2764], a187);
      double a188 = 0.0;
      a188 = fma(0.83 * r1delt, ws[2496], a188);
      lu[2991] = a143;
      lu[2992] = a182;
      lu[2993] = a187;
      lu[2994] = a188;
      vd[54] = 1.0 / a54;
    }
}
__device__ __noinline__ void gear_pdecomp_s1_0_1(double* __restrict__ ws, double r1delt)
{
    double* __restrict__ lu = ws + 3484;
    double* __restrict__ vd = ws + 6769;
    { // row 55
      double a39 = 0.0;
      a39 = fma(0.619 * r1delt, ws[2529], a39);
      double a55 = 1.0;
      a55 = fma(-r1delt, ws[2533], a55);
      a55 = fma(-r1delt, ws[2629], a55);
      double a86 = 0.0;
      double a92 = 0.0;
      a92 = fma(0.584 * r1delt, ws[2531], a92);
      double a162 = 0.0;
      double a186 = 0.0;
      a186 = fma(-r1delt, ws[2630], a186);
      double a188 = 0.0;
      a188 = fma(0.619 * r1delt, ws[2530], a188);
      a188 = fma(0.584 * r1delt, ws[2532], a188);
      a188 = fma(-r1delt, ws[2534], a188);
      a39 = a39 * CHEM_LDLU(vd + 39);
      lu[12] = a39;
      a86 = fma(-a39, CHEM_LDLU(lu + 3044), a86);
      a162 = fma(-a39, CHEM_LDLU(lu + 3045), a162);
      a186 = fma(-a39, CHEM_LDLU(lu + 3046), a186);
      a188 = fma(-a39, CHEM_LDLU(lu + 3047), a188);
      lu[2986] = a86;
      lu[2987] = a92;
      lu[2988] = a162;
      lu[2989] = a186;
      lu[2990] = a188;
      vd[55] = 1.0 / a55;
    }
    { // row 56
      double a56 = 1.0;
      a56 = fma(-r1delt, ws[2551], a56);
      double a110 = 0.0;
      a110 = fma(r1delt, ws[2777], a110);
      double a146 = 0.0;
      a146 = fma(r1delt, ws[2775], a146);
      double a187 = 0.0;
      a187 = fma(r1delt, ws[2776], a187);
      a187 = fma(r1delt, ws[2778], a187);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[2552], a188);
      lu[2982] = a110;
      lu[2983] = a146;
      lu[2984] = a187;
      lu[2985] = a188;
      vd[56] = 1.0 / a56;
    }
    { // row 57
      double a57 = 1.0;
      a57 = fma(-r1delt, ws[2563], a57);
      a57 = fma(-r1delt, ws[2631], a57);
      a57 = fma(-r1delt, ws[1504], a57);
      double a146 = 0.0;
      a146 = fma(r1delt, ws[2637], a146);
      double a185 = 0.0;
      a185 = fma(r1delt, ws[2638], a185);
      double a186 = 0.0;
      a186 = fma(-r1delt, ws[2632], a186);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[2564], a188);
      lu[2978] = a146;
      lu[2979] = a185;
      lu[2980] = a186;
      lu[2981] = a188;
      vd[57] = 1.0 / a57;
    }
    { // row 58
      double a58 = 1.0;
      a58 = fma(-r1delt, ws[3083], a58);
      a58 = fma(-r1delt, ws[3085], a58);
      double a99 = 0.0;
      a99 = fma(0.51 * r1delt, ws[3081], a99);
      double a182 = 0.0;
      a182 = fma(-r1delt, ws[3084], a182);
      double a187 = 0.0;
      a187 = fma(-r1delt, ws[3086], a187);
      double a188 = 0.0;
      a188 = fma(0.51 * r1delt, ws[3082], a188);
      lu[2974] = a99;
      lu[2975] = a182;
      lu[2976] = a187;
      lu[2977] = a188;
      vd[58] = 1.0 / a58;
    }
    { // row 59
      double a36 = 0.0;
      a36 = fma(0.01 * r1delt, ws[2575], a36);
      double a59 = 1.0;
      a59 = fma(-r1delt, ws[2443], a59);
      double a86 = 0.0;
      a86 = fma(0.02 * r1delt, ws[2573], a86);
      double a162 = 0.0;
      a162 = fma(0.02 * r1delt, ws[2574], a162);
      a162 = fma(0.01 * r1delt, ws[2576], a162);
      double a186 = 0.0;
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[2444], a188);
      a36 = a36 * CHEM_LDLU(vd + 36);
      lu[13] = a36;
      a162 = fma(-a36, CHEM_LDLU(lu + 3054), a162);
      a186 = fma(-a36, CHEM_LDLU(lu + 3055), a186);
      a188 = fma(-a36, CHEM_LDLU(lu + 3056), a188);
      lu[2970] = a86;
      lu[2971] = a162;
      lu[2972] = a186;
      lu[2973] = a188;
      vd[59] = 1.0 / a59;
    }
    { // row 60
      double a50 = 0.0;
      a50 = fma(r1delt, ws[3095], a50);
      double a60 = 1.0;
      a60 = fma(-r1delt, ws[3097], a60);
      a60 = fma(-r1delt, ws[3099], a60);
      a60 = fma(-r1delt, ws[3101], a60);
      double a162 = 0.0;
      double a182 = 0.0;
      a182 = fma(-r1delt, ws[3100], a182);
      double a186 = 0.0;
      a186 = fma(r1delt, ws[3096], a186);
      a186 = fma(-r1delt, ws[3102], a186);
      double a187 = 0.0;
      a187 = fma(-r1delt, ws[3098], a187);
      double a188 = 0.0;
      a50 = a50 * CHEM_LDLU(vd + 50);
      lu[14] = a50;
      a162 = fma(-a50, CHEM_LDLU(lu + 3010), a162);
      a186 = fma(-a50, CHEM_LDLU(lu + 3011), a186);
      a188 = fma(-a50, CHEM_LDLU(lu + 3012), a188);
      lu[2965] = a162;
      lu[2966] = a182;
      lu[2967] = a186;
      lu[2968] = a187;
      lu[2969] = a188;
      vd[60] = 1.0 / a60;
    }
    { // row 61
      double a61 = 1.0;
      a61 = fma(-r1delt, ws[1783], a61);
      a61 = fma(-r1delt, ws[3171], a61);
      a61 = fma(-r1delt, ws[3185], a61);
      a61 = fma(-r1delt, ws[3199], a61);
      double a74 = 0.0;
      a74 = fma(0.72 * r1delt, ws[3129], a74);
      a74 = fma(r1delt, ws[3143], a74);
      double a182 = 0.0;
      a182 = fma(0.72 * r1delt, ws[3130], a182);
      a182 = fma(-r1delt, ws[3172], a182);
      double a186 = 0.0;
      a186 = fma(r1delt, ws[3144], a186);
      a186 = fma(-r1delt, ws[3186], a186);
      double a187 = 0.0;
      a187 = fma(-r1delt, ws[3200], a187);
      lu[2961] = a74;
      lu[2962] = a182;
      lu[2963] = a186;
      lu[2964] = a187;
      vd[61] = 1.0 / a61;
    }
    { // row 62
      double a62 = 1.0;
      a62 = fma(-r1delt, ws[1784], a62);
      a62 = fma(-r1delt, ws[3173], a62);
      a62 = fma(-r1delt, ws[3187], a62);
      a62 = fma(-r1delt, ws[3201], a62);
      double a75 = 0.0;
      a75 = fma(0.72 * r1delt, ws[3131], a75);
      a75 = fma(r1delt, ws[3145], a75);
      double a182 = 0.0;
      a182 = fma(0.72 * r1delt, ws[3132], a182);
      a182 = fma(-r1delt, ws[3174], a182);
      double a186 = 0.0;
      a186 = fma(r1delt, ws[3146], a186);
      a186 = fma(-r1delt, ws[3188], a186);
      double a187 = 0.0;
      a187 = fma(-r1delt, ws[3202], a187);
      lu[2957] = a75;
      lu[2958] = a182;
      lu[2959] = a186;
      lu[2960] = a187;
      vd[62] = 1.0 / a62;
    }
    { // row 63
      double a63 = 1.0;
      a63 = fma(-r1delt, ws[1785], a63);
      a63 = fma(-r1delt, ws[3175], a63);
      a63 = fma(-r1delt, ws[3189], a63);
      a63 = fma(-r1delt, ws[3203], a63);
      double a76 = 0.0;
      a76 = fma(0.72 * r1delt, ws[3133], a76);
      a76 = fma(r1delt, ws[3147], a76);
      double a182 = 0.0;
      a182 = fma(0.72 * r1delt, ws[3134], a182);
      a182 = fma(-r1delt, ws[3176], a182);
      double a186 = 0.0;
      a186 = fma(r1delt, ws[3148], a186);
      a186 = fma(-r1delt, ws[3190], a186);
      double a187 = 0.0;
      a187 = fma(-r1delt, ws[3204], a187);
      lu[2953] = a76;
      lu[2954] = a182;
      lu[2955] = a186;
      lu[2956] = a187;
      vd[63] = 1.0 / a63;
    }
    { // row 64
      double a64 = 1.0;
      a64 = fma(-r1delt, ws[1786], a64);
      a64 = fma(-r1delt, ws[3177], a64);
      a64 = fma(-r1delt, ws[3191], a64);
      a64 = fma(-r1delt, ws[3205], a64);
      double a77 = 0.0;
      a77 = fma(0.72 * r1delt, ws[3135], a77);
      a77 = fma(r1delt, ws[3149], a77);
      double a182 = 0.0;
      a182 = fma(0.72 * r1delt, ws[3136], a182);
      a182 = fma(-r1delt, ws[3178], a182);
      double a186 = 0.0;
      a186 = fma(r1delt, ws[3150], a186);
      a186 = fma(-r1delt, ws[3192], a186);
      double a187 = 0.0;
      a187 = fma(-r1delt, ws[3206], a187);
      lu[2949] = a77;
      lu[2950] = a182;
      lu[2951] = a186;
      lu[2952] = a187;
      vd[64] = 1.0 / a64;
    }
    { // row 65
      double a65 = 1.0;
      a65 = fma(-r1delt, ws[1787], a65);
      a65 = fma(-r1delt, ws[3179], a65);
      a65 = fma(-r1delt, ws[3193], a65);
      a65 = fma(-r1delt, ws[3207], a65);
      double a78 = 0.0;
      a78 = fma(0.72 * r1delt, ws[3137], a78);
      a78 = fma(r1delt, ws[3151], a78);
      double a182 = 0.0;
      a182 = fma(0.72 * r1delt, ws[3138], a182);
      a182 = fma(-r1delt, ws[3180], a182);
      double a186 = 0.0;
      a186 = fma(r1delt, ws[3152], a186);
      a186 = fma(-r1delt, ws[3194], a186);
      double a187 = 0.0;
      a187 = fma(-r1delt, ws[3208], a187);
      lu[2945] = a78;
      lu[2946] = a182;
      lu[2947] = a186;
      lu[2948] = a187;
      vd[65] = 1.0 / a65;
    }
    { // row 66
      double a66 = 1.0;
      a66 = fma(-r1delt, ws[1788], a66);
      a66 = fma(-r1delt, ws[3181], a66);
      a66 = fma(-r1delt, ws[3195], a66);
      a66 = fma(-r1delt, ws[3209], a66);
      double a79 = 0.0;
      a79 = fma(0.72 * r1delt, ws[3139], a79);
      a79 = fma(r1delt, ws[3153], a79);
      double a182 = 0.0;
      a182 = fma(0.72 * r1delt, ws[3140], a182);
      a182 = fma(-r1delt, ws[3182], a182);
      double a186 = 0.0;
      a186 = fma(r1delt, ws[3154], a186);
      a186 = fma(-r1delt, ws[3196], a186);
      double a187 = 0.0;
      a187 = fma(-r1delt, ws[3210], a187);
      lu[2941] = a79;
      lu[2942] = a182;
      lu[2943] = a186;
      lu[2944] = a187;
      vd[66] = 1.0 / a66;
    }
    { // row 67
      double a67 = 1.0;
      a67 = fma(-r1delt, ws[1789], a67);
      a67 = fma(-r1delt, ws[3183], a67);
      a67 = fma(-r1delt, ws[3197], a67);
      a67 = fma(-r1delt, ws[3211], a67);
      double a122 = 0.0;
      a122 = fma(0.74 * r1delt, ws[3141], a122);
      a122 = fma(r1delt, ws[3155], a122);
      double a182 = 0.0;
      a182 = fma(0.74 * r1delt, ws[3142], a182);
      a182 = fma(-r1delt, ws[3184], a182);
      double a186 = 0.0;
      a186 = fma(r1delt, ws[3156], a186);
      a186 = fma(-r1delt, ws[3198], a186);
      double a187 = 0.0;
      a187 = fma(-r1delt, ws[3212], a187);
      lu[2937] = a122;
      lu[2938] = a182;
      lu[2939] = a186;
      lu[2940] = a187;
      vd[67] = 1.0 / a67;
    }
    { // row 68
      double a36 = 0.0;
      a36 = fma(0.01 * r1delt, ws[2575], a36);
      double a44 = 0.0;
      a44 = fma(0.0665 * r1delt, ws[2577], a44);
      double a68 = 1.0;
      a68 = fma(-r1delt, ws[2445], a68);
      double a86 = 0.0;
      a86 = fma(0.015 * r1delt, ws[2573], a86);
      double a162 = 0.0;
      a162 = fma(0.015 * r1delt, ws[2574], a162);
      a162 = fma(0.01 * r1delt, ws[2576], a162);
      a162 = fma(0.0665 * r1delt, ws[2578], a162);
      double a186 = 0.0;
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[2446], a188);
      a36 = a36 * CHEM_LDLU(vd + 36);
      lu[15] = a36;
      a162 = fma(-a36, CHEM_LDLU(lu + 3054), a162);
      a186 = fma(-a36, CHEM_LDLU(lu + 3055), a186);
      a188 = fma(-a36, CHEM_LDLU(lu + 3056), a188);
      a44 = a44 * CHEM_LDLU(vd + 44);
      lu[16] = a44;
      a162 = fma(-a44, CHEM_LDLU(lu + 3028), a162);
      a186 = fma(-a44, CHEM_LDLU(lu + 3029), a186);
      a188 = fma(-a44, CHEM_LDLU(lu + 3030), a188);
      lu[2933] = a86;
      lu[2934] = a162;
      lu[2935] = a186;
      lu[2936] = a188;
      vd[68] = 1.0 / a68;
    }
    { // row 69
      double a51 = 0.0;
      a51 = fma(0.95 * r1delt, ws[2479], a51);
      a51 = fma(0.65 * r1delt, ws[2481], a51);
      double a69 = 1.0;
      a69 = fma(-r1delt, ws[2486], a69);
      a69 = fma(-r1delt, ws[1754], a69);
      double a87 = 0.0;
      a87 = fma(0.35 * r1delt, ws[2483], a87);
      double a162 = 0.0;
      double a182 = 0.0;
      a182 = fma(0.65 * r1delt, ws[2482], a182);
      double a186 = 0.0;
      double a187 = 0.0;
      a187 = fma(0.95 * r1delt, ws[2480], a187);
      double a188 = 0.0;
      a188 = fma(0.35 * r1delt, ws[2484], a188);
      a188 = fma(-r1delt, ws[2485], a188);
      a51 = a51 * CHEM_LDLU(vd + 51);
      lu[17] = a51;
      a162 = fma(-a51, CHEM_LDLU(lu + 3005), a162);
      a182 = fma(-a51, CHEM_LDLU(lu + 3006), a182);
      a186 = fma(-a51, CHEM_LDLU(lu + 3007), a186);
      a187 = fma(-a51, CHEM_LDLU(lu + 3008), a187);
      a188 = fma(-a51, CHEM_LDLU(lu + 3009), a188);
      lu[2927] = a87;
      lu[2928] = a162;
      lu[2929] = a182;
      lu[2930] = a186;
      lu[2931] = a187;
      lu[2932] = a188;
      vd[69] = 1.0 / a69;
    }
    { // row 70
      double a49 = 0.0;
      a49 = fma(0.17 * r1delt, ws[3077], a49);
      double a70 = 1.0;
      a70 = fma(-r1delt, ws[2449], a70);
      a70 = fma(-r1delt, ws[2571], a70);
      a70 = fma(-r1delt, ws[2599], a70);
      double a111 = 0.0;
      a111 = fma(0.25 * r1delt, ws[1718], a111);
      double a162 = 0.0;
      a162 = fma(-r1delt, ws[2572], a162);
      a162 = fma(0.17 * r1delt, ws[3078], a162);
      double a186 = 0.0;
      a186 = fma(-r1delt, ws[2600], a186);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[2450], a188);
      a49 = a49 * CHEM_LDLU(vd + 49);
      lu[18] = a49;
      a162 = fma(-a49, CHEM_LDLU(lu + 3013), a162);
      a186 = fma(-a49, CHEM_LDLU(lu + 3014), a186);
      a188 = fma(-a49, CHEM_LDLU(lu + 3015), a188);
      lu[2923] = a111;
      lu[2924] = a162;
      lu[2925] = a186;
      lu[2926] = a188;
      vd[70] = 1.0 / a70;
    }
    { // row 71
      double a71 = 1.0;
      a71 = fma(-r1delt, ws[2701], a71);
      a71 = fma(-r1delt, ws[2859], a71);
      a71 = fma(-r1delt, ws[2933], a71);
      a71 = fma(-r1delt, ws[3003], a71);
      double a81 = 0.0;
      a81 = fma(r1delt, ws[2699], a81);
      a81 = fma(r1delt, ws[2857], a81);
      a81 = fma(r1delt, ws[2931], a81);
      a81 = fma(r1delt, ws[3001], a81);
      double a181 = 0.0;
      a181 = fma(r1delt, ws[2932], a181);
      a181 = fma(-r1delt, ws[2934], a181);
      double a182 = 0.0;
      a182 = fma(r1delt, ws[2700], a182);
      a182 = fma(-r1delt, ws[2702], a182);
      double a184 = 0.0;
      a184 = fma(r1delt, ws[2858], a184);
      a184 = fma(-r1delt, ws[2860], a184);
      double a186 = 0.0;
      a186 = fma(r1delt, ws[3002], a186);
      a186 = fma(-r1delt, ws[3004], a186);
      lu[2918] = a81;
      lu[2919] = a181;
      lu[2920] = a182;
      lu[2921] = a184;
      lu[2922] = a186;
      vd[71] = 1.0 / a71;
    }
    { // row 72
      double a50 = 0.0;
      a50 = fma(r1delt, ws[3105], a50);
      double a72 = 1.0;
      a72 = fma(-r1delt, ws[3107], a72);
      a72 = fma(-r1delt, ws[3109], a72);
      a72 = fma(-r1delt, ws[3111], a72);
      double a162 = 0.0;
      double a182 = 0.0;
      a182 = fma(-r1delt, ws[3112], a182);
      double a186 = 0.0;
      a186 = fma(-r1delt, ws[3110], a186);
      double a187 = 0.0;
      a187 = fma(-r1delt, ws[3108], a187);
      double a188 = 0.0;
      a188 = fma(r1delt, ws[3106], a188);
      a50 = a50 * CHEM_LDLU(vd + 50);
      lu[19] = a50;
      a162 = fma(-a50, CHEM_LDLU(lu + 3010), a162);
      a186 = fma(-a50, CHEM_LDLU(lu + 3011), a186);
      a188 = fma(-a50, CHEM_LDLU(lu + 3012), a188);
      lu[2913] = a162;
      lu[2914] = a182;
      lu[2915] = a186;
      lu[2916] = a187;
      lu[2917] = a188;
      vd[72] = 1.0 / a72;
    }
    { // row 73
      double a18 = 0.0;
      a18 = fma(r1delt, ws[1369], a18);
      a18 = fma(r1delt, ws[1370], a18);
      double a73 = 1.0;
      a73 = fma(-r1delt, ws[1367], a73);
      a73 = fma(-r1delt, ws[2393], a73);
      a73 = fma(-r1delt, ws[2404], a73);
      a73 = fma(-r1delt, ws[2416], a73);
      a73 = fma(-r1delt, ws[2418], a73);
      double a162 = 0.0;
      a162 = fma(r1delt, ws[1323], a162);
      a162 = fma(-r1delt, ws[2394], a162);
      double a182 = 0.0;
      a182 = fma(-r1delt, ws[2403], a182);
      double a185 = 0.0;
      a185 = fma(r1delt, ws[1326], a185);
      a185 = fma(-r1delt, ws[2415], a185);
      a185 = fma(-r1delt, ws[2417], a185);
      double a186 = 0.0;
      a186 = fma(r1delt, ws[1328], a186);
      a18 = a18 * CHEM_LDLU(vd + 18);
      lu[20] = a18;
      a162 = fma(-a18, CHEM_LDLU(lu + 3078), a162);
      lu[2909] = a162;
      lu[2910] = a182;
      lu[2911] = a185;
      lu[2912] = a186;
      vd[73] = 1.0 / a73;
    }
    { // row 74
      double a19 = 0.0;
      a19 = fma(r1delt, ws[3115], a19);
      double a74 = 1.0;
      a74 = fma(-r1delt, ws[3129], a74);
      a74 = fma(-r1delt, ws[3143], a74);
      a74 = fma(-r1delt, ws[3157], a74);
      double a182 = 0.0;
      a182 = fma(-r1delt, ws[3130], a182);
      double a186 = 0.0;
      a186 = fma(-r1delt, ws[3144], a186);
      double a187 = 0.0;
      a187 = fma(-r1delt, ws[3158], a187);
      double a188 = 0.0;
      a188 = fma(r1delt, ws[3116], a188);
      a19 = a19 * CHEM_LDLU(vd + 19);
      lu[21] = a19;
      a188 = fma(-a19, CHEM_LDLU(lu + 3077), a188);
      lu[2905] = a182;
      lu[2906] = a186;
      lu[2907] = a187;
      lu[2908] = a188;
      vd[74] = 1.0 / a74;
    }
    { // row 75
      double a20 = 0.0;
      a20 = fma(r1delt, ws[3117], a20);
      double a75 = 1.0;
      a75 = fma(-r1delt, ws[3131], a75);
      a75 = fma(-r1delt, ws[3145], a75);
      a75 = fma(-r1delt, ws[3159], a75);
      double a182 = 0.0;
      a182 = fma(-r1delt, ws[3132], a182);
      double a186 = 0.0;
      a186 = fma(-r1delt, ws[3146], a186);
      double a187 = 0.0;
      a187 = fma(-r1delt, ws[3160], a187);
      double a188 = 0.0;
      a188 = fma(r1delt, ws[3118], a188);
      a20 = a20 * CHEM_LDLU(vd + 20);
      lu[22] = a20;
      a188 = fma(-a20, CHEM_LDLU(lu + 3076), a188);
      lu[2901] = a182;
      lu[2902] = a186;
      lu[2903] = a187;
      lu[2904] = a188;
      vd[75] = 1.0 / a75;
    }
    { // row 76
      double a21 = 0.0;
      a21 = fma(r1delt, ws[3119], a21);
      double a76 = 1.0;
      a76 = fma(-r1delt, ws[3133], a76);
      a76 = fma(-r1delt, ws[3147], a76);
      a76 = fma(-r1delt, ws[3161], a76);
      double a182 = 0.0;
      a182 = fma(-r1delt, ws[3134], a182);
      double a186 = 0.0;
      a186 = fma(-r1delt, ws[3148], a186);
      double a187 = 0.0;
      a187 = fma(-r1delt, ws[3162], a187);
      double a188 = 0.0;
      a188 = fma(r1delt, ws[3120], a188);
      a21 = a21 * CHEM_LDLU(vd + 21);
      lu[23] = a21;
      a188 = fma(-a21, CHEM_LDLU(lu + 3075), a188);
      lu[2897] = a182;
      lu[2898] = a186;
      lu[2899] = a187;
      lu[2900] = a188;
      vd[76] = 1.0 / a76;
    }
    { // row 77
      double a22 = 0.0;
      a22 = fma(r1delt, ws[3121], a22);
      double a77 = 1.0;
      a77 = fma(-r1delt, ws[3135], a77);
      a77 = fma(-r1delt, ws[3149], a77);
      a77 = fma(-r1delt, ws[3163], a77);
      double a182 = 0.0;
      a182 = fma(-r1delt, ws[3136], a182);
      double a186 = 0.0;
      a186 = fma(-r1delt, ws[3150], a186);
      double a187 = 0.0;
      a187 = fma(-r1delt, ws[3164], a187);
      double a188 = 0.0;
      a188 = fma(r1delt, ws[3122], a188);
      a22 = a22 * CHEM_LDLU(vd + 22);
      lu[24] = a22;
      a188 = fma(-a22, CHEM_LDLU(lu + 3074), a188);
      lu[2893] = a182;
      lu[2894] = a186;
      lu[2895] = a187;
      lu[2896] = a188;
      vd[77] = 1.0 / a77;
    }
    { // row 78
      double a23 = 0.0;
      a23 = fma(r1delt, ws[3123], a23);
      double a78 = 1.0;
      a78 = fma(-r1delt, ws[3137], a78);
      a78 = fma(-r1delt, ws[3151], a78);
      a78 = fma(-r1delt, ws[3165], a78);
      double a182 = 0.0;
      a182 = fma(-r1delt, ws[3138], a182);
      double a186 = 0.0;
      a186 = fma(-r1delt, ws[3152], a186);
      double a187 = 0.0;
      a187 = fma(-r1delt, ws[3166], a187);
      double a188 = 0.0;
      a188 = fma(r1delt, ws[3124], a188);
      a23 = a23 * CHEM_LDLU(vd + 23);
      lu[25] = a23;
      a188 = fma(-a23, CHEM_LDLU(lu + 3073), a188);
      lu[2889] = a182;
      lu[2890] = a186;
      lu[2891] = a187;
      lu[2892] = a188;
      vd[78] = 1.0 / a78;
    }
    { // row 79
      double a24 = 0.0;
      a24 = fma(r1delt, ws[3125], a24);
      double a79 = 1.0;
      a79 = fma(-r1delt, ws[3139], a79);
      a79 = fma(-r1delt, ws[3153], a79);
      a79 = fma(-r1delt, ws[3167], a79);
      double a182 = 0.0;
      a182 = fma(-r1delt, ws[3140], a182);
      double a186 = 0.0;
      a186 = fma(-r1delt, ws[3154], a186);
      double a187 = 0.0;
      a187 = fma(-r1delt, ws[3168], a187);
      double a188 = 0.0;
      a188 = fma(r1delt, ws[3126], a188);
      a24 = a24 * CHEM_LDLU(vd + 24);
      lu[26] = a24;
      a188 = fma(-a24, CHEM_LDLU(lu + 3072), a188);
      lu[2885] = a182;
      lu[2886] = a186;
      lu[2887] = a187;
      lu[2888] = a188;
      vd[79] = 1.0 / a79;
    }
    { // row 80
      double a44 = 0.0;
      a44 = fma(0.2145 * r1delt, ws[2577], a44);
      double a80 = 1.0;
      a80 = fma(-r1delt, ws[1497], a80);
      a80 = fma(-r1delt, ws[2677], a80);
      a80 = fma(-r1delt, ws[2761], a80);
      double a142 = 0.0;
      a142 = fma(0.23 * r1delt, ws[2493], a142);
      double a162 = 0.0;
      a162 = fma(0.2145 * r1delt, ws[2578], a162);
      double a182 = 0.0;
      a182 = fma(-r1delt, ws[2678], a182);
      double a186 = 0.0;
      double a187 = 0.0;
      a187 = fma(-r1delt, ws[2762], a187);
      double a188 = 0.0;
      a188 = fma(0.23 * r1delt, ws[2494], a188);
      a44 = a44 * CHEM_LDLU(vd + 44);
      lu[27] = a44;
      a162 = fma(-a44, CHEM_LDLU(lu + 3028), a162);
      a186 = fma(-a44, CHEM_LDLU(lu + 3029), a186);
      a188 = fma(-a44, CHEM_LDLU(lu + 3030), a188);
      lu[2879] = a142;
      lu[2880] = a162;
      lu[2881] = a182;
      lu[2882] = a186;
      lu[2883] = a187;
      lu[2884] = a188;
      vd[80] = 1.0 / a80;
    }
    { // row 81
      double a81 = 1.0;
      a81 = fma(-r1delt, ws[2699], a81);
      a81 = fma(-r1delt, ws[2857], a81);
      a81 = fma(-r1delt, ws[2931], a81);
      a81 = fma(-r1delt, ws[3001], a81);
      double a139 = 0.0;
      a139 = fma(r1delt, ws[2527], a139);
      double a181 = 0.0;
      a181 = fma(-r1delt, ws[2932], a181);
      double a182 = 0.0;
      a182 = fma(-r1delt, ws[2700], a182);
      double a184 = 0.0;
      a184 = fma(-r1delt, ws[2858], a184);
      double a186 = 0.0;
      a186 = fma(-r1delt, ws[3002], a186);
      double a188 = 0.0;
      a188 = fma(r1delt, ws[2528], a188);
      lu[2873] = a139;
      lu[2874] = a181;
      lu[2875] = a182;
      lu[2876] = a184;
      lu[2877] = a186;
      lu[2878] = a188;
      vd[81] = 1.0 / a81;
    }
}
__device__ __noinline__ void gear_pdecomp_s1_0_2(double* __restrict__ ws, double r1delt)
{
    double* __restrict__ lu = ws + 3484;
    double* __restrict__ vd = ws + 6769;
    { // row 82
      double a44 = 0.0;
      a44 = fma(0.975 * r1delt, ws[2605], a44);
      double a82 = 1.0;
      a82 = fma(-r1delt, ws[2665], a82);
      a82 = fma(-r1delt, ws[2749], a82);
      a82 = fma(-r1delt, ws[2827], a82);
      a82 = fma(-r1delt, ws[2901], a82);
      a82 = fma(-r1delt, ws[2979], a82);
      double a162 = 0.0;
      double a181 = 0.0;
      a181 = fma(-r1delt, ws[2902], a181);
      double a182 = 0.0;
      a182 = fma(-r1delt, ws[2666], a182);
      double a184 = 0.0;
      a184 = fma(-r1delt, ws[2828], a184);
      double a186 = 0.0;
      a186 = fma(0.975 * r1delt, ws[2606], a186);
      a186 = fma(-r1delt, ws[2980], a186);
      double a187 = 0.0;
      a187 = fma(-r1delt, ws[2750], a187);
      double a188 = 0.0;
      a44 = a44 * CHEM_LDLU(vd + 44);
      lu[28] = a44;
      a162 = fma(-a44, CHEM_LDLU(lu + 3028), a162);
      a186 = fma(-a44, CHEM_LDLU(lu + 3029), a186);
      a188 = fma(-a44, CHEM_LDLU(lu + 3030), a188);
      lu[2866] = a162;
      lu[2867] = a181;
      lu[2868] = a182;
      lu[2869] = a184;
      lu[2870] = a186;
      lu[2871] = a187;
      lu[2872] = a188;
      vd[82] = 1.0 / a82;
    }
    { // row 83
      double a45 = 0.0;
      a45 = fma(0.945 * r1delt, ws[2607], a45);
      double a83 = 1.0;
      a83 = fma(-r1delt, ws[2673], a83);
      a83 = fma(-r1delt, ws[2757], a83);
      a83 = fma(-r1delt, ws[2835], a83);
      a83 = fma(-r1delt, ws[2909], a83);
      a83 = fma(-r1delt, ws[2981], a83);
      double a162 = 0.0;
      double a181 = 0.0;
      a181 = fma(-r1delt, ws[2910], a181);
      double a182 = 0.0;
      a182 = fma(-r1delt, ws[2674], a182);
      double a184 = 0.0;
      a184 = fma(-r1delt, ws[2836], a184);
      double a186 = 0.0;
      a186 = fma(0.945 * r1delt, ws[2608], a186);
      a186 = fma(-r1delt, ws[2982], a186);
      double a187 = 0.0;
      a187 = fma(-r1delt, ws[2758], a187);
      double a188 = 0.0;
      a45 = a45 * CHEM_LDLU(vd + 45);
      lu[29] = a45;
      a162 = fma(-a45, CHEM_LDLU(lu + 3025), a162);
      a186 = fma(-a45, CHEM_LDLU(lu + 3026), a186);
      a188 = fma(-a45, CHEM_LDLU(lu + 3027), a188);
      lu[2859] = a162;
      lu[2860] = a181;
      lu[2861] = a182;
      lu[2862] = a184;
      lu[2863] = a186;
      lu[2864] = a187;
      lu[2865] = a188;
      vd[83] = 1.0 / a83;
    }
    { // row 84
      double a71 = 0.0;
      a71 = fma(r1delt, ws[2701], a71);
      a71 = fma(r1delt, ws[2859], a71);
      a71 = fma(r1delt, ws[2933], a71);
      a71 = fma(r1delt, ws[3003], a71);
      double a81 = 0.0;
      double a84 = 1.0;
      a84 = fma(-r1delt, ws[2717], a84);
      double a139 = 0.0;
      double a181 = 0.0;
      a181 = fma(r1delt, ws[2934], a181);
      double a182 = 0.0;
      a182 = fma(r1delt, ws[2702], a182);
      double a184 = 0.0;
      a184 = fma(r1delt, ws[2860], a184);
      double a185 = 0.0;
      a185 = fma(-r1delt, ws[2718], a185);
      double a186 = 0.0;
      a186 = fma(r1delt, ws[3004], a186);
      double a188 = 0.0;
      a71 = a71 * CHEM_LDLU(vd + 71);
      lu[30] = a71;
      a81 = fma(-a71, CHEM_LDLU(lu + 2918), a81);
      a181 = fma(-a71, CHEM_LDLU(lu + 2919), a181);
      a182 = fma(-a71, CHEM_LDLU(lu + 2920), a182);
      a184 = fma(-a71, CHEM_LDLU(lu + 2921), a184);
      a186 = fma(-a71, CHEM_LDLU(lu + 2922), a186);
      a81 = a81 * CHEM_LDLU(vd + 81);
      lu[31] = a81;
      a139 = fma(-a81, CHEM_LDLU(lu + 2873), a139);
      a181 = fma(-a81, CHEM_LDLU(lu + 2874), a181);
      a182 = fma(-a81, CHEM_LDLU(lu + 2875), a182);
      a184 = fma(-a81, CHEM_LDLU(lu + 2876), a184);
      a186 = fma(-a81, CHEM_LDLU(lu + 2877), a186);
      a188 = fma(-a81, CHEM_LDLU(lu + 2878), a188);
      lu[2852] = a139;
      lu[2853] = a181;
      lu[2854] = a182;
      lu[2855] = a184;
      lu[2856] = a185;
      lu[2857] = a186;
      lu[2858] = a188;
      vd[84] = 1.0 / a84;
    }
    { // row 85
      double a85 = 1.0;
      double a116 = 0.0;
      a116 = fma(0.04 * r1delt, ws[3047], a116);
      a116 = fma(0.04 * r1delt, ws[3049], a116);
      a116 = fma(0.04 * r1delt, ws[3051], a116);
      double a117 = 0.0;
      a117 = fma(0.04 * r1delt, ws[3029], a117);
      a117 = fma(0.04 * r1delt, ws[3031], a117);
      a117 = fma(0.04 * r1delt, ws[3033], a117);
      double a120 = 0.0;
      a120 = fma(0.04 * r1delt, ws[3041], a120);
      a120 = fma(0.04 * r1delt, ws[3043], a120);
      a120 = fma(0.04 * r1delt, ws[3045], a120);
      double a123 = 0.0;
      a123 = fma(0.04 * r1delt, ws[3035], a123);
      a123 = fma(0.04 * r1delt, ws[3037], a123);
      a123 = fma(0.04 * r1delt, ws[3039], a123);
      double a130 = 0.0;
      a130 = fma(0.04 * r1delt, ws[3030], a130);
      a130 = fma(0.04 * r1delt, ws[3036], a130);
      a130 = fma(0.04 * r1delt, ws[3042], a130);
      a130 = fma(0.04 * r1delt, ws[3048], a130);
      double a131 = 0.0;
      a131 = fma(0.04 * r1delt, ws[3032], a131);
      a131 = fma(0.04 * r1delt, ws[3038], a131);
      a131 = fma(0.04 * r1delt, ws[3044], a131);
      a131 = fma(0.04 * r1delt, ws[3050], a131);
      double a134 = 0.0;
      a134 = fma(0.04 * r1delt, ws[3034], a134);
      a134 = fma(0.04 * r1delt, ws[3040], a134);
      a134 = fma(0.04 * r1delt, ws[3046], a134);
      a134 = fma(0.04 * r1delt, ws[3052], a134);
      lu[2845] = a116;
      lu[2846] = a117;
      lu[2847] = a120;
      lu[2848] = a123;
      lu[2849] = a130;
      lu[2850] = a131;
      lu[2851] = a134;
      vd[85] = 1.0 / a85;
    }
    { // row 86
      double a41 = 0.0;
      a41 = fma(0.153 * r1delt, ws[2465], a41);
      double a86 = 1.0;
      a86 = fma(-r1delt, ws[2451], a86);
      a86 = fma(-r1delt, ws[2573], a86);
      a86 = fma(-r1delt, ws[2601], a86);
      double a98 = 0.0;
      a98 = fma(0.25 * r1delt, ws[3073], a98);
      double a162 = 0.0;
      a162 = fma(0.153 * r1delt, ws[2466], a162);
      a162 = fma(-r1delt, ws[2574], a162);
      double a184 = 0.0;
      a184 = fma(0.25 * r1delt, ws[3074], a184);
      double a186 = 0.0;
      a186 = fma(-r1delt, ws[2602], a186);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[2452], a188);
      a41 = a41 * CHEM_LDLU(vd + 41);
      lu[32] = a41;
      a162 = fma(-a41, CHEM_LDLU(lu + 3038), a162);
      a186 = fma(-a41, CHEM_LDLU(lu + 3039), a186);
      a188 = fma(-a41, CHEM_LDLU(lu + 3040), a188);
      lu[2840] = a98;
      lu[2841] = a162;
      lu[2842] = a184;
      lu[2843] = a186;
      lu[2844] = a188;
      vd[86] = 1.0 / a86;
    }
    { // row 87
      double a41 = 0.0;
      a41 = fma(0.045 * r1delt, ws[2467], a41);
      double a51 = 0.0;
      a51 = fma(0.05 * r1delt, ws[2481], a51);
      double a87 = 1.0;
      a87 = fma(-r1delt, ws[2483], a87);
      a87 = fma(-r1delt, ws[1423], a87);
      double a134 = 0.0;
      a134 = fma(0.13 * r1delt, ws[2473], a134);
      double a162 = 0.0;
      double a182 = 0.0;
      a182 = fma(0.13 * r1delt, ws[2474], a182);
      a182 = fma(0.05 * r1delt, ws[2482], a182);
      double a186 = 0.0;
      a186 = fma(0.045 * r1delt, ws[2468], a186);
      double a187 = 0.0;
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[2484], a188);
      a41 = a41 * CHEM_LDLU(vd + 41);
      lu[33] = a41;
      a162 = fma(-a41, CHEM_LDLU(lu + 3038), a162);
      a186 = fma(-a41, CHEM_LDLU(lu + 3039), a186);
      a188 = fma(-a41, CHEM_LDLU(lu + 3040), a188);
      a51 = a51 * CHEM_LDLU(vd + 51);
      lu[34] = a51;
      a162 = fma(-a51, CHEM_LDLU(lu + 3005), a162);
      a182 = fma(-a51, CHEM_LDLU(lu + 3006), a182);
      a186 = fma(-a51, CHEM_LDLU(lu + 3007), a186);
      a187 = fma(-a51, CHEM_LDLU(lu + 3008), a187);
      a188 = fma(-a51, CHEM_LDLU(lu + 3009), a188);
      lu[2834] = a134;
      lu[2835] = a162;
      lu[2836] = a182;
      lu[2837] = a186;
      lu[2838] = a187;
      lu[2839] = a188;
      vd[87] = 1.0 / a87;
    }
    { // row 88
      double a44 = 0.0;
      a44 = fma(0.0385 * r1delt, ws[2577], a44);
      double a88 = 1.0;
      a88 = fma(-r1delt, ws[1353], a88);
      a88 = fma(-r1delt, ws[2543], a88);
      double a143 = 0.0;
      a143 = fma(0.23 * r1delt, ws[2581], a143);
      double a162 = 0.0;
      a162 = fma(0.0385 * r1delt, ws[2578], a162);
      a162 = fma(0.23 * r1delt, ws[2582], a162);
      double a184 = 0.0;
      a184 = fma(r1delt, ws[2723], a184);
      double a186 = 0.0;
      double a187 = 0.0;
      a187 = fma(r1delt, ws[2724], a187);
      double a188 = 0.0;
      a188 = fma(-r1delt, ws[2544], a188);
      a44 = a44 * CHEM_LDLU(vd + 44);
      lu[35] = a44;
      a162 = fma(-a44, CHEM_LDLU(lu + 3028), a162);
      a186 = fma(-a44, CHEM_LDLU(lu + 3029), a186);
      a188 = fma(-a44, CHEM_LDLU(lu + 3030), a188);
      lu[2828] = a143;
      lu[2829] = a162;
      lu[2830] = a184;
      lu[2831] = a186;
      lu[2832] = a187;
      lu[2833] = a188;
      vd[88] = 1.0 / a88;
    }
    { // row 89
      double a89 = 1.0;
      a89 = fma(-r1delt, ws[2685], a89);
      a89 = fma(-r1delt, ws[2769], a89);
      a89 = fma(-r1delt, ws[2843], a89);
      a89 = fma(-r1delt, ws[2917], a89);
      a89 = fma(-r1delt, ws[2987], a89);
      double a140 = 0.0;
      a140 = fma(r1delt, ws[2503], a140);
      double a181 = 0.0;
      a181 = fma(-r1delt, ws[2918], a181);
      double a182 = 0.0;
      a182 = fma(-r1delt, ws[2686], a182);
      double a184 = 0.0;
      a184 = fma(-r1delt, ws[2844], a184);
      double a186 = 0.0;
      a186 = fma(-r1delt, ws[2988], a186);
      double a187 = 0.0;
      a187 = fma(-r1delt, ws[2770], a187);
      double a188 = 0.0;
      a188 = fma(r1delt, ws[2504], a188);
      lu[2821] = a140;
      lu[2822] = a181;
      lu[2823] = a182;
      lu[2824] = a184;
      lu[2825] = a186;
      lu[2826] = a187;
      lu[2827] = a188;
      vd[89] = 1.0 / a89;
    }
    { // row 90
      double a90 = 1.0;
      a90 = fma(-r1delt, ws[2695], a90);
      a90 = fma(-r1delt, ws[2779], a90);
      a90 = fma(-r1delt, ws[2853], a90);
      a90 = fma(-r1delt, ws[2927], a90);
      a90 = fma(-r1delt, ws[2997], a90);
      double a148 = 0.0;
      a148 = fma(r1delt, ws[2513], a148);
      double a181 = 0.0;
      a181 = fma(-r1delt, ws[2928], a181);
      double a182 = 0.0;
      a182 = fma(-r1delt, ws[2696], a182);
      double a184 = 0.0;
      a184 = fma(-r1delt, ws[2854], a184);
      double a186 = 0.0;
      a186 = fma(-r1delt, ws[2998], a186);
      double a187 = 0.0;
      a187 = fma(-r1delt, ws[2780], a187);
      double a188 = 0.0;
      a188 = fma(r1delt, ws[2514], a188);
      lu[2814] = a148;
      lu[2815] = a181;
      lu[2816] = a182;
      lu[2817] = a184;
      lu[2818] = a186;
      lu[2819] = a187;
      lu[2820] = a188;
      vd[90] = 1.0 / a90;
    }
    { // row 91
      double a91 = 1.0;
      a91 = fma(-r1delt, ws[2697], a91);
      a91 = fma(-r1delt, ws[2781], a91);
      a91 = fma(-r1delt, ws[2855], a91);
      a91 = fma(-r1delt, ws[2929], a91);
      a91 = fma(-r1delt, ws[2999], a91);
      double a121 = 0.0;
      a121 = fma(0.687 * r1delt, ws[2515], a121);
      double a181 = 0.0;
      a181 = fma(-r1delt, ws[2930], a181);
      double a182 = 0.0;
      a182 = fma(-r1delt, ws[2698], a182);
      double a184 = 0.0;
      a184 = fma(-r1delt, ws[2856], a184);
      double a186 = 0.0;
      a186 = fma(-r1delt, ws[3000], a186);
      double a187 = 0.0;
      a187 = fma(-r1delt, ws[2782], a187);
      double a188 = 0.0;
      a188 = fma(0.687 * r1delt, ws[2516], a188);
      lu[2807] = a121;
      lu[2808] = a181;
      lu[2809] = a182;
      lu[2810] = a184;
      lu[2811] = a186;
      lu[2812] = a187;
      lu[2813] = a188;
      vd[91] = 1.0 / a91;
    }
    { // row 92
      double a9 = 0.0;
      a9 = fma(0.18 * r1delt, ws[2459], a9);
      double a10 = 0.0;
      a10 = fma(0.17 * r1delt, ws[2461], a10);
      double a11 = 0.0;
      a11 = fma(0.18 * r1delt, ws[2463], a11);
      double a92 = 1.0;
      a92 = fma(-r1delt, ws[2531], a92);
      a92 = fma(-r1delt, ws[2627], a92);
      double a101 = 0.0;
      a101 = fma(r1delt, ws[2785], a101);
      double a186 = 0.0;
      a186 = fma(-r1delt, ws[2628], a186);
      double a187 = 0.0;
      a187 = fma(r1delt, ws[2786], a187);
      double a188 = 0.0;
      a188 = fma(0.18 * r1delt, ws[2460], a188);
      a188 = fma(0.17 * r1delt, ws[2462], a188);
      a188 = fma(0.18 * r1delt, ws[2464], a188);
      a188 = fma(-r1delt, ws[2532], a188);
      a9 = a9 * CHEM_LDLU(vd + 9);
      lu[36] = a9;
      a188 = fma(-a9, CHEM_LDLU(lu + 3088), a188);
      a10 = a10 * CHEM_LDLU(vd + 10);
      lu[37] = a10;
      a188 = fma(-a10, CHEM_LDLU(lu + 3087), a188);
      a11 = a11 * CHEM_LDLU(vd + 11);
      lu[38] = a11;
      a188 = fma(-a11, CHEM_LDLU(lu + 3086), a188);
      lu[2803] = a101;
      lu[2804] = a186;
      lu[2805] = a187;
      lu[2806] = a188;
      vd[92] = 1.0 / a92;
    }
    { // row 93
      double a93 = 1.0;
      a93 = fma(-r1delt, ws[2707], a93);
      a93 = fma(-r1delt, ws[2789], a93);
      a93 = fma(-r1delt, ws[2865], a93);
      a93 = fma(-r1delt, ws[2939], a93);
      a93 = fma(-r1delt, ws[3009], a93);
      double a178 = 0.0;
      a178 = fma(0.36 * r1delt, ws[2555], a178);
      double a181 = 0.0;
      a181 = fma(-r1delt, ws[2940], a181);
      double a182 = 0.0;
      a182 = fma(-r1delt, ws[2708], a182);
      double a184 = 0.0;
      a184 = fma(-r1delt, ws[2866], a184);
      double a186 = 0.0;
      a186 = fma(-r1delt, ws[3010], a186);
      double a187 = 0.0;
      a187 = fma(-r1delt, ws[2790], a187);
      double a188 = 0.0;
      a188 = fma(0.36 * r1delt, ws[2556], a188);
      lu[2796] = a178;
      lu[2797] = a181;
      lu[2798] = a182;
      lu[2799] = a184;
      lu[2800] = a186;
      lu[2801] = a187;
      lu[2802] = a188;
      vd[93] = 1.0 / a93;
    }
    { // row 94
      double a70 = 0.0;
      a70 = fma(r1delt, ws[2449], a70);
      double a94 = 1.0;
      a94 = fma(-r1delt, ws[2647], a94);
      a94 = fma(-r1delt, ws[2731], a94);
      a94 = fma(-r1delt, ws[2807], a94);
      a94 = fma(-r1delt, ws[2881], a94);
      a94 = fma(-r1delt, ws[2959], a94);
      double a111 = 0.0;
      double a162 = 0.0;
      double a181 = 0.0;
      a181 = fma(-r1delt, ws[2882], a181);
      double a182 = 0.0;
      a182 = fma(-r1delt, ws[2648], a182);
      double a184 = 0.0;
      a184 = fma(-r1delt, ws[2808], a184);
      double a186 = 0.0;
      a186 = fma(-r1delt, ws[2960], a186);
      double a187 = 0.0;
      a187 = fma(-r1delt, ws[2732], a187);
      double a188 = 0.0;
      a188 = fma(r1delt, ws[2450], a188);
      a70 = a70 * CHEM_LDLU(vd + 70);
      lu[39] = a70;
      a111 = fma(-a70, CHEM_LDLU(lu + 2923), a111);
      a162 = fma(-a70, CHEM_LDLU(lu + 2924), a162);
      a186 = fma(-a70, CHEM_LDLU(lu + 2925), a186);
      a188 = fma(-a70, CHEM_LDLU(lu + 2926), a188);
      lu[2788] = a111;
      lu[2789] = a162;
      lu[2790] = a181;
      lu[2791] = a182;
      lu[2792] = a184;
      lu[2793] = a186;
      lu[2794] = a187;
      lu[2795] = a188;
      vd[94] = 1.0 / a94;
    }
    { // row 95
      double a95 = 1.0;
      a95 = fma(-r1delt, ws[2705], a95);
      a95 = fma(-r1delt, ws[2787], a95);
      a95 = fma(-r1delt, ws[2863], a95);
      a95 = fma(-r1delt, ws[2937], a95);
      a95 = fma(-r1delt, ws[3007], a95);
      double a119 = 0.0;
      a119 = fma(r1delt, ws[2597], a119);
      double a162 = 0.0;
      a162 = fma(r1delt, ws[2598], a162);
      double a181 = 0.0;
      a181 = fma(-r1delt, ws[2938], a181);
      double a182 = 0.0;
      a182 = fma(-r1delt, ws[2706], a182);
      double a184 = 0.0;
      a184 = fma(-r1delt, ws[2864], a184);
      double a186 = 0.0;
      a186 = fma(-r1delt, ws[3008], a186);
      double a187 = 0.0;
      a187 = fma(-r1delt, ws[2788], a187);
      lu[2781] = a119;
      lu[2782] = a162;
      lu[2783] = a181;
      lu[2784] = a182;
      lu[2785] = a184;
      lu[2786] = a186;
      lu[2787] = a187;
      vd[95] = 1.0 / a95;
    }
    { // row 96
      double a39 = 0.0;
      a39 = fma(0.424 * r1delt, ws[2625], a39);
      double a86 = 0.0;
      double a92 = 0.0;
      a92 = fma(0.4 * r1delt, ws[2627], a92);
      double a96 = 1.0;
      a96 = fma(-r1delt, ws[2713], a96);
      a96 = fma(-r1delt, ws[2795], a96);
      a96 = fma(-r1delt, ws[2871], a96);
      a96 = fma(-r1delt, ws[2945], a96);
      a96 = fma(-r1delt, ws[3015], a96);
      double a98 = 0.0;
      double a101 = 0.0;
      double a162 = 0.0;
      double a181 = 0.0;
      a181 = fma(-r1delt, ws[2946], a181);
      double a182 = 0.0;
      a182 = fma(-r1delt, ws[2714], a182);
      double a184 = 0.0;
      a184 = fma(-r1delt, ws[2872], a184);
      double a186 = 0.0;
      a186 = fma(0.424 * r1delt, ws[2626], a186);
      a186 = fma(0.4 * r1delt, ws[2628], a186);
      a186 = fma(-r1delt, ws[3016], a186);
      double a187 = 0.0;
      a187 = fma(-r1delt, ws[2796], a187);
      double a188 = 0.0;
      a39 = a39 * CHEM_LDLU(vd + 39);
      lu[40] = a39;
      a86 = fma(-a39, CHEM_LDLU(lu + 3044), a86);
      a162 = fma(-a39, CHEM_LDLU(lu + 3045), a162);
      a186 = fma(-a39, CHEM_LDLU(lu + 3046), a186);
      a188 = fma(-a39, CHEM_LDLU(lu + 3047), a188);
      a86 = a86 * CHEM_LDLU(vd + 86);
      lu[41] = a86;
      a98 = fma(-a86, CHEM_LDLU(lu + 2840), a98);
      a162 = fma(-a86, CHEM_LDLU(lu + 2841), a162);
      a184 = fma(-a86, CHEM_LDLU(lu + 2842), a184);
      a186 = fma(-a86, CHEM_LDLU(lu + 2843), a186);
      a188 = fma(-a86, CHEM_LDLU(lu + 2844), a188);
      a92 = a92 * CHEM_LDLU(vd + 92);
      lu[42] = a92;
      a101 = fma(-a92, CHEM_LDLU(lu + 2803), a101);
      a186 = fma(-a92, CHEM_LDLU(lu + 2804), a186);
      a187 = fma(-a92, CHEM_LDLU(lu + 2805), a187);
      a188 = fma(-a92, CHEM_LDLU(lu + 2806), a188);
      lu[2772] = a98;
      lu[2773] = a101;
      lu[2774] = a162;
      lu[2775] = a181;
      lu[2776] = a182;
      lu[2777] = a184;
      lu[2778] = a186;
      lu[2779] = a187;
      lu[2780] = a188;
      vd[96] = 1.0 / a96;
    }
    { // row 97
      double a10 = 0.0;
      a10 = fma(0.83 * r1delt, ws[2461], a10);
      double a97 = 1.0;
      a97 = fma(-r1delt, ws[2657], a97);
      a97 = fma(-r1delt, ws[2741], a97);
      a97 = fma(-r1delt, ws[2817], a97);
      a97 = fma(-r1delt, ws[2891], a97);
      a97 = fma(-r1delt, ws[2969], a97);
      double a181 = 0.0;
      a181 = fma(-r1delt, ws[2892], a181);
      double a182 = 0.0;
      a182 = fma(-r1delt, ws[2658], a182);
      double a184 = 0.0;
      a184 = fma(-r1delt, ws[2818], a184);
      double a186 = 0.0;
      a186 = fma(-r1delt, ws[2970], a186);
      double a187 = 0.0;
      a187 = fma(-r1delt, ws[2742], a187);
      double a188 = 0.0;
      a188 = fma(0.83 * r1delt, ws[2462], a188);
      a10 = a10 * CHEM_LDLU(vd + 10);
      lu[43] = a10;
      a188 = fma(-a10, CHEM_LDLU(lu + 3087), a188);
      lu[2766] = a181;
      lu[2767] = a182;
      lu[2768] = a184;
      lu[2769] = a186;
      lu[2770] = a187;
      lu[2771] = a188;
      vd[97] = 1.0 / a97;
    }
}
}  // namespace mech_cracmm2
