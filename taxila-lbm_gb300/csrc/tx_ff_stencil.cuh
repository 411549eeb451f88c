/* Generated by oracle/ff_stencil_parse.py from the reference's lbm_forcing.F90
 * (LBMAddFluidFluidForcesD3 :51-958, LBMAddFluidFluidForcesD2 :960-1299).
 * One row per gradient term in the reference's accumulation order:
 *   e      neighbour offset; the term adds (e_d * w) * (psi(x+e) - psi(x)) to
 *          grad_d and (e_d^2 * w) to weightsum_d for every axis with e_d != 0;
 *   w      index into the isotropy weight vector ffw (1-based);
 *   level  4, 8 or 10: the term is used when isotropy_order >= level;
 *   naux/aux  path cells between x and x+e; bit b of truth is set when the
 *          term is taken with aux cell q pore space iff bit q of b is set
 *          (x+e itself must always be pore space). */
#pragma once
namespace tx {
struct FFTerm { int e[3]; int w; int level; int naux; int aux[4][3]; unsigned truth; };
constexpr int FF_D3_COUNT = 92;
__host__ __device__ constexpr FFTerm ff_d3(int t) {
  switch (t) {
    case 0: return FFTerm{{1, 0, 0}, 1, 4, 0, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x1u};  // lbm_forcing.F90:85
    case 1: return FFTerm{{-1, 0, 0}, 1, 4, 0, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x1u};  // lbm_forcing.F90:90
    case 2: return FFTerm{{0, 1, 0}, 1, 4, 0, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x1u};  // lbm_forcing.F90:95
    case 3: return FFTerm{{0, -1, 0}, 1, 4, 0, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x1u};  // lbm_forcing.F90:100
    case 4: return FFTerm{{0, 0, 1}, 1, 4, 0, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x1u};  // lbm_forcing.F90:105
    case 5: return FFTerm{{0, 0, -1}, 1, 4, 0, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x1u};  // lbm_forcing.F90:110
    case 6: return FFTerm{{1, 1, 0}, 2, 4, 0, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x1u};  // lbm_forcing.F90:117
    case 7: return FFTerm{{-1, 1, 0}, 2, 4, 0, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x1u};  // lbm_forcing.F90:125
    case 8: return FFTerm{{1, -1, 0}, 2, 4, 0, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x1u};  // lbm_forcing.F90:133
    case 9: return FFTerm{{-1, -1, 0}, 2, 4, 0, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x1u};  // lbm_forcing.F90:141
    case 10: return FFTerm{{1, 0, 1}, 2, 4, 0, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x1u};  // lbm_forcing.F90:151
    case 11: return FFTerm{{-1, 0, 1}, 2, 4, 0, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x1u};  // lbm_forcing.F90:159
    case 12: return FFTerm{{1, 0, -1}, 2, 4, 0, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x1u};  // lbm_forcing.F90:167
    case 13: return FFTerm{{-1, 0, -1}, 2, 4, 0, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x1u};  // lbm_forcing.F90:175
    case 14: return FFTerm{{0, 1, 1}, 2, 4, 0, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x1u};  // lbm_forcing.F90:185
    case 15: return FFTerm{{0, -1, 1}, 2, 4, 0, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x1u};  // lbm_forcing.F90:193
    case 16: return FFTerm{{0, 1, -1}, 2, 4, 0, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x1u};  // lbm_forcing.F90:201
    case 17: return FFTerm{{0, -1, -1}, 2, 4, 0, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x1u};  // lbm_forcing.F90:209
    case 18: return FFTerm{{1, 1, 1}, 3, 8, 0, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x1u};  // lbm_forcing.F90:224
    case 19: return FFTerm{{-1, 1, 1}, 3, 8, 0, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x1u};  // lbm_forcing.F90:235
    case 20: return FFTerm{{-1, -1, 1}, 3, 8, 0, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x1u};  // lbm_forcing.F90:246
    case 21: return FFTerm{{1, -1, 1}, 3, 8, 0, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x1u};  // lbm_forcing.F90:257
    case 22: return FFTerm{{1, 1, -1}, 3, 8, 0, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x1u};  // lbm_forcing.F90:268
    case 23: return FFTerm{{-1, 1, -1}, 3, 8, 0, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x1u};  // lbm_forcing.F90:279
    case 24: return FFTerm{{-1, -1, -1}, 3, 8, 0, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x1u};  // lbm_forcing.F90:290
    case 25: return FFTerm{{1, -1, -1}, 3, 8, 0, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x1u};  // lbm_forcing.F90:301
    case 26: return FFTerm{{2, 0, 0}, 4, 8, 1, {{1, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x2u};  // lbm_forcing.F90:314
    case 27: return FFTerm{{-2, 0, 0}, 4, 8, 1, {{-1, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x2u};  // lbm_forcing.F90:319
    case 28: return FFTerm{{0, 2, 0}, 4, 8, 1, {{0, 1, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x2u};  // lbm_forcing.F90:324
    case 29: return FFTerm{{0, -2, 0}, 4, 8, 1, {{0, -1, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x2u};  // lbm_forcing.F90:329
    case 30: return FFTerm{{0, 0, 2}, 4, 8, 1, {{0, 0, 1}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x2u};  // lbm_forcing.F90:334
    case 31: return FFTerm{{0, 0, -2}, 4, 8, 1, {{0, 0, -1}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x2u};  // lbm_forcing.F90:339
    case 32: return FFTerm{{2, 1, 0}, 5, 8, 2, {{1, 1, 0}, {1, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0xeu};  // lbm_forcing.F90:346
    case 33: return FFTerm{{-2, 1, 0}, 5, 8, 2, {{-1, 1, 0}, {-1, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0xeu};  // lbm_forcing.F90:354
    case 34: return FFTerm{{-2, -1, 0}, 5, 8, 2, {{-1, -1, 0}, {-1, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0xeu};  // lbm_forcing.F90:362
    case 35: return FFTerm{{2, -1, 0}, 5, 8, 2, {{1, -1, 0}, {1, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0xeu};  // lbm_forcing.F90:370
    case 36: return FFTerm{{2, 0, 1}, 5, 8, 2, {{1, 0, 1}, {1, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0xeu};  // lbm_forcing.F90:378
    case 37: return FFTerm{{-2, 0, 1}, 5, 8, 2, {{-1, 0, 1}, {-1, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0xeu};  // lbm_forcing.F90:386
    case 38: return FFTerm{{-2, 0, -1}, 5, 8, 2, {{-1, 0, -1}, {-1, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0xeu};  // lbm_forcing.F90:394
    case 39: return FFTerm{{2, 0, -1}, 5, 8, 2, {{1, 0, -1}, {1, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0xeu};  // lbm_forcing.F90:402
    case 40: return FFTerm{{1, 2, 0}, 5, 8, 2, {{1, 1, 0}, {0, 1, 0}, {0, 0, 0}, {0, 0, 0}}, 0xeu};  // lbm_forcing.F90:412
    case 41: return FFTerm{{-1, 2, 0}, 5, 8, 2, {{-1, 1, 0}, {0, 1, 0}, {0, 0, 0}, {0, 0, 0}}, 0xeu};  // lbm_forcing.F90:420
    case 42: return FFTerm{{-1, -2, 0}, 5, 8, 2, {{-1, -1, 0}, {0, -1, 0}, {0, 0, 0}, {0, 0, 0}}, 0xeu};  // lbm_forcing.F90:428
    case 43: return FFTerm{{1, -2, 0}, 5, 8, 2, {{1, -1, 0}, {0, -1, 0}, {0, 0, 0}, {0, 0, 0}}, 0xeu};  // lbm_forcing.F90:436
    case 44: return FFTerm{{0, 2, 1}, 5, 8, 2, {{0, 1, 1}, {0, 1, 0}, {0, 0, 0}, {0, 0, 0}}, 0xeu};  // lbm_forcing.F90:444
    case 45: return FFTerm{{0, -2, 1}, 5, 8, 2, {{0, -1, 1}, {0, -1, 0}, {0, 0, 0}, {0, 0, 0}}, 0xeu};  // lbm_forcing.F90:452
    case 46: return FFTerm{{0, 2, -1}, 5, 8, 2, {{0, 1, -1}, {0, 1, 0}, {0, 0, 0}, {0, 0, 0}}, 0xeu};  // lbm_forcing.F90:460
    case 47: return FFTerm{{0, -2, -1}, 5, 8, 2, {{0, -1, -1}, {0, -1, 0}, {0, 0, 0}, {0, 0, 0}}, 0xeu};  // lbm_forcing.F90:468
    case 48: return FFTerm{{1, 0, 2}, 5, 8, 2, {{1, 0, 1}, {0, 0, 1}, {0, 0, 0}, {0, 0, 0}}, 0xeu};  // lbm_forcing.F90:478
    case 49: return FFTerm{{0, 1, 2}, 5, 8, 2, {{0, 1, 1}, {0, 0, 1}, {0, 0, 0}, {0, 0, 0}}, 0xeu};  // lbm_forcing.F90:486
    case 50: return FFTerm{{-1, 0, 2}, 5, 8, 2, {{-1, 0, 1}, {0, 0, 1}, {0, 0, 0}, {0, 0, 0}}, 0xeu};  // lbm_forcing.F90:494
    case 51: return FFTerm{{0, -1, 2}, 5, 8, 2, {{0, -1, 1}, {0, 0, 1}, {0, 0, 0}, {0, 0, 0}}, 0xeu};  // lbm_forcing.F90:502
    case 52: return FFTerm{{1, 0, -2}, 5, 8, 2, {{1, 0, -1}, {0, 0, -1}, {0, 0, 0}, {0, 0, 0}}, 0xeu};  // lbm_forcing.F90:511
    case 53: return FFTerm{{0, 1, -2}, 5, 8, 2, {{0, 1, -1}, {0, 0, -1}, {0, 0, 0}, {0, 0, 0}}, 0xeu};  // lbm_forcing.F90:519
    case 54: return FFTerm{{-1, 0, -2}, 5, 8, 2, {{-1, 0, -1}, {0, 0, -1}, {0, 0, 0}, {0, 0, 0}}, 0xeu};  // lbm_forcing.F90:527
    case 55: return FFTerm{{0, -1, -2}, 5, 8, 2, {{0, -1, -1}, {0, 0, -1}, {0, 0, 0}, {0, 0, 0}}, 0xeu};  // lbm_forcing.F90:535
    case 56: return FFTerm{{2, 1, 1}, 6, 8, 4, {{1, 1, 0}, {1, 0, 0}, {1, 1, 1}, {1, 0, 1}}, 0xfffeu};  // lbm_forcing.F90:546
    case 57: return FFTerm{{-2, 1, 1}, 6, 8, 4, {{-1, 1, 0}, {-1, 0, 0}, {-1, 1, 1}, {-1, 0, 1}}, 0xfffeu};  // lbm_forcing.F90:558
    case 58: return FFTerm{{-2, -1, 1}, 6, 8, 4, {{-1, -1, 0}, {-1, 0, 0}, {-1, -1, 1}, {-1, 0, 1}}, 0xfffeu};  // lbm_forcing.F90:570
    case 59: return FFTerm{{2, -1, 1}, 6, 8, 4, {{1, -1, 0}, {1, 0, 0}, {1, -1, 1}, {1, 0, 1}}, 0xfffeu};  // lbm_forcing.F90:582
    case 60: return FFTerm{{2, 1, -1}, 6, 8, 4, {{1, 1, 0}, {1, 0, 0}, {1, 1, -1}, {1, 0, -1}}, 0xfffeu};  // lbm_forcing.F90:594
    case 61: return FFTerm{{-2, 1, -1}, 6, 8, 4, {{-1, 1, 0}, {-1, 0, 0}, {-1, 1, -1}, {-1, 0, -1}}, 0xfffeu};  // lbm_forcing.F90:606
    case 62: return FFTerm{{-2, -1, -1}, 6, 8, 4, {{-1, -1, 0}, {-1, 0, 0}, {-1, -1, -1}, {-1, 0, -1}}, 0xfffeu};  // lbm_forcing.F90:618
    case 63: return FFTerm{{2, -1, -1}, 6, 8, 4, {{1, -1, 0}, {1, 0, 0}, {1, -1, -1}, {1, 0, -1}}, 0xfffeu};  // lbm_forcing.F90:630
    case 64: return FFTerm{{1, 2, 1}, 6, 8, 4, {{1, 1, 0}, {0, 1, 0}, {1, 1, 1}, {0, 1, 1}}, 0xfffeu};  // lbm_forcing.F90:644
    case 65: return FFTerm{{-1, 2, 1}, 6, 8, 4, {{-1, 1, 0}, {0, 1, 0}, {-1, 1, 1}, {0, 1, 1}}, 0xfffeu};  // lbm_forcing.F90:656
    case 66: return FFTerm{{-1, -2, 1}, 6, 8, 4, {{-1, -1, 0}, {0, -1, 0}, {-1, -1, 1}, {0, -1, 1}}, 0xfffeu};  // lbm_forcing.F90:668
    case 67: return FFTerm{{1, -2, 1}, 6, 8, 4, {{1, -1, 0}, {0, -1, 0}, {1, -1, 1}, {0, -1, 1}}, 0xfffeu};  // lbm_forcing.F90:680
    case 68: return FFTerm{{1, 2, -1}, 6, 8, 4, {{1, 1, 0}, {0, 1, 0}, {1, 1, -1}, {0, 1, -1}}, 0xfffeu};  // lbm_forcing.F90:692
    case 69: return FFTerm{{-1, -2, -1}, 6, 8, 4, {{-1, -1, 0}, {0, -1, 0}, {-1, -1, -1}, {0, -1, -1}}, 0xfffeu};  // lbm_forcing.F90:704
    case 70: return FFTerm{{-1, 2, -1}, 6, 8, 4, {{-1, 1, 0}, {0, 1, 0}, {-1, 1, -1}, {0, 1, -1}}, 0xfffeu};  // lbm_forcing.F90:716
    case 71: return FFTerm{{1, -2, -1}, 6, 8, 4, {{1, -1, 0}, {0, -1, 0}, {1, -1, -1}, {0, -1, -1}}, 0xfffeu};  // lbm_forcing.F90:728
    case 72: return FFTerm{{1, 1, 2}, 6, 8, 4, {{1, 1, 1}, {0, 0, 1}, {1, 0, 1}, {0, 1, 1}}, 0xfffeu};  // lbm_forcing.F90:742
    case 73: return FFTerm{{-1, 1, 2}, 6, 8, 4, {{-1, 1, 1}, {0, 0, 1}, {-1, 0, 1}, {0, 1, 1}}, 0xfffeu};  // lbm_forcing.F90:754
    case 74: return FFTerm{{-1, -1, 2}, 6, 8, 4, {{-1, -1, 1}, {0, 0, 1}, {-1, 0, 1}, {0, -1, 1}}, 0xfffeu};  // lbm_forcing.F90:766
    case 75: return FFTerm{{1, -1, 2}, 6, 8, 4, {{1, -1, 1}, {0, 0, 1}, {1, 0, 1}, {0, -1, 1}}, 0xfffeu};  // lbm_forcing.F90:778
    case 76: return FFTerm{{1, 1, -2}, 6, 8, 4, {{1, 1, -1}, {0, 0, -1}, {1, 0, -1}, {0, 1, -1}}, 0xfffeu};  // lbm_forcing.F90:790
    case 77: return FFTerm{{-1, 1, -2}, 6, 8, 4, {{-1, 1, -1}, {0, 0, -1}, {-1, 0, -1}, {0, 1, -1}}, 0xfffeu};  // lbm_forcing.F90:802
    case 78: return FFTerm{{-1, -1, -2}, 6, 8, 4, {{-1, -1, -1}, {0, 0, -1}, {-1, 0, -1}, {0, -1, -1}}, 0xfffeu};  // lbm_forcing.F90:814
    case 79: return FFTerm{{1, -1, -2}, 6, 8, 4, {{1, -1, -1}, {0, 0, -1}, {1, 0, -1}, {0, -1, -1}}, 0xfffeu};  // lbm_forcing.F90:826
    case 80: return FFTerm{{2, 2, 0}, 8, 8, 1, {{1, 1, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x2u};  // lbm_forcing.F90:840
    case 81: return FFTerm{{-2, 2, 0}, 8, 8, 1, {{-1, 1, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x2u};  // lbm_forcing.F90:848
    case 82: return FFTerm{{-2, -2, 0}, 8, 8, 1, {{-1, -1, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x2u};  // lbm_forcing.F90:856
    case 83: return FFTerm{{2, -2, 0}, 8, 8, 1, {{1, -1, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x2u};  // lbm_forcing.F90:864
    case 84: return FFTerm{{2, 0, 2}, 8, 8, 1, {{1, 0, 1}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x2u};  // lbm_forcing.F90:874
    case 85: return FFTerm{{-2, 0, 2}, 8, 8, 1, {{-1, 0, 1}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x2u};  // lbm_forcing.F90:882
    case 86: return FFTerm{{-2, 0, -2}, 8, 8, 1, {{-1, 0, -1}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x2u};  // lbm_forcing.F90:890
    case 87: return FFTerm{{2, 0, -2}, 8, 8, 1, {{1, 0, -1}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x2u};  // lbm_forcing.F90:898
    case 88: return FFTerm{{0, 2, 2}, 8, 8, 1, {{0, 1, 1}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x2u};  // lbm_forcing.F90:908
    case 89: return FFTerm{{0, -2, 2}, 8, 8, 1, {{0, -1, 1}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x2u};  // lbm_forcing.F90:916
    case 90: return FFTerm{{0, -2, -2}, 8, 8, 1, {{0, -1, -1}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x2u};  // lbm_forcing.F90:924
    case 91: return FFTerm{{0, 2, -2}, 8, 8, 1, {{0, 1, -1}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x2u};  // lbm_forcing.F90:932
    default: return FFTerm{{0, 0, 0}, 0, 0, 0, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0u};
  }
}
constexpr int FF_D2_COUNT = 36;
__host__ __device__ constexpr FFTerm ff_d2(int t) {
  switch (t) {
    case 0: return FFTerm{{1, 0, 0}, 1, 4, 0, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x1u};  // lbm_forcing.F90:994
    case 1: return FFTerm{{-1, 0, 0}, 1, 4, 0, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x1u};  // lbm_forcing.F90:999
    case 2: return FFTerm{{0, 1, 0}, 1, 4, 0, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x1u};  // lbm_forcing.F90:1004
    case 3: return FFTerm{{0, -1, 0}, 1, 4, 0, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x1u};  // lbm_forcing.F90:1009
    case 4: return FFTerm{{1, 1, 0}, 2, 4, 0, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x1u};  // lbm_forcing.F90:1016
    case 5: return FFTerm{{-1, 1, 0}, 2, 4, 0, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x1u};  // lbm_forcing.F90:1024
    case 6: return FFTerm{{1, -1, 0}, 2, 4, 0, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x1u};  // lbm_forcing.F90:1032
    case 7: return FFTerm{{-1, -1, 0}, 2, 4, 0, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x1u};  // lbm_forcing.F90:1040
    case 8: return FFTerm{{2, 0, 0}, 4, 8, 1, {{1, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x2u};  // lbm_forcing.F90:1054
    case 9: return FFTerm{{-2, 0, 0}, 4, 8, 1, {{-1, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x2u};  // lbm_forcing.F90:1059
    case 10: return FFTerm{{0, 2, 0}, 4, 8, 1, {{0, 1, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x2u};  // lbm_forcing.F90:1064
    case 11: return FFTerm{{0, -2, 0}, 4, 8, 1, {{0, -1, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x2u};  // lbm_forcing.F90:1069
    case 12: return FFTerm{{2, 1, 0}, 5, 8, 2, {{1, 1, 0}, {1, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0xeu};  // lbm_forcing.F90:1076
    case 13: return FFTerm{{2, -1, 0}, 5, 8, 2, {{1, -1, 0}, {1, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0xeu};  // lbm_forcing.F90:1084
    case 14: return FFTerm{{-2, 1, 0}, 5, 8, 2, {{-1, 1, 0}, {-1, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0xeu};  // lbm_forcing.F90:1092
    case 15: return FFTerm{{-2, -1, 0}, 5, 8, 2, {{-1, -1, 0}, {-1, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0xeu};  // lbm_forcing.F90:1100
    case 16: return FFTerm{{1, 2, 0}, 5, 8, 2, {{1, 1, 0}, {0, 1, 0}, {0, 0, 0}, {0, 0, 0}}, 0xeu};  // lbm_forcing.F90:1108
    case 17: return FFTerm{{1, -2, 0}, 5, 8, 2, {{1, -1, 0}, {0, -1, 0}, {0, 0, 0}, {0, 0, 0}}, 0xeu};  // lbm_forcing.F90:1116
    case 18: return FFTerm{{-1, 2, 0}, 5, 8, 2, {{-1, 1, 0}, {0, 1, 0}, {0, 0, 0}, {0, 0, 0}}, 0xeu};  // lbm_forcing.F90:1124
    case 19: return FFTerm{{-1, -2, 0}, 5, 8, 2, {{-1, -1, 0}, {0, -1, 0}, {0, 0, 0}, {0, 0, 0}}, 0xeu};  // lbm_forcing.F90:1132
    case 20: return FFTerm{{2, 2, 0}, 8, 8, 1, {{1, 1, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x2u};  // lbm_forcing.F90:1142
    case 21: return FFTerm{{-2, 2, 0}, 8, 8, 1, {{-1, 1, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x2u};  // lbm_forcing.F90:1150
    case 22: return FFTerm{{2, -2, 0}, 8, 8, 1, {{1, -1, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x2u};  // lbm_forcing.F90:1158
    case 23: return FFTerm{{-2, -2, 0}, 8, 8, 1, {{-1, -1, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x2u};  // lbm_forcing.F90:1166
    case 24: return FFTerm{{3, 0, 0}, 9, 10, 2, {{2, 0, 0}, {1, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x8u};  // lbm_forcing.F90:1181
    case 25: return FFTerm{{-3, 0, 0}, 9, 10, 2, {{-2, 0, 0}, {-1, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0x8u};  // lbm_forcing.F90:1186
    case 26: return FFTerm{{0, 3, 0}, 9, 10, 2, {{0, 2, 0}, {0, 1, 0}, {0, 0, 0}, {0, 0, 0}}, 0x8u};  // lbm_forcing.F90:1191
    case 27: return FFTerm{{0, -3, 0}, 9, 10, 2, {{0, -2, 0}, {0, -1, 0}, {0, 0, 0}, {0, 0, 0}}, 0x8u};  // lbm_forcing.F90:1196
    case 28: return FFTerm{{3, 1, 0}, 10, 10, 4, {{1, 0, 0}, {2, 0, 0}, {1, 1, 0}, {2, 1, 0}}, 0xf888u};  // lbm_forcing.F90:1203
    case 29: return FFTerm{{3, -1, 0}, 10, 10, 4, {{1, 0, 0}, {2, 0, 0}, {1, -1, 0}, {2, -1, 0}}, 0xf888u};  // lbm_forcing.F90:1213
    case 30: return FFTerm{{-3, 1, 0}, 10, 10, 4, {{-1, 0, 0}, {-2, 0, 0}, {-1, 1, 0}, {-2, 1, 0}}, 0xf888u};  // lbm_forcing.F90:1223
    case 31: return FFTerm{{-3, -1, 0}, 10, 10, 4, {{-1, 0, 0}, {-2, 0, 0}, {-1, -1, 0}, {-2, -1, 0}}, 0xf888u};  // lbm_forcing.F90:1233
    case 32: return FFTerm{{1, 3, 0}, 10, 10, 4, {{0, 1, 0}, {0, 2, 0}, {1, 1, 0}, {1, 2, 0}}, 0xf888u};  // lbm_forcing.F90:1243
    case 33: return FFTerm{{1, -3, 0}, 10, 10, 4, {{0, -1, 0}, {0, -2, 0}, {1, -1, 0}, {1, -2, 0}}, 0xf888u};  // lbm_forcing.F90:1253
    case 34: return FFTerm{{-1, 3, 0}, 10, 10, 4, {{0, 1, 0}, {0, 2, 0}, {-1, 1, 0}, {-1, 2, 0}}, 0xf888u};  // lbm_forcing.F90:1263
    case 35: return FFTerm{{-1, -3, 0}, 10, 10, 4, {{0, -1, 0}, {0, -2, 0}, {-1, -1, 0}, {-1, -2, 0}}, 0xf888u};  // lbm_forcing.F90:1273
    default: return FFTerm{{0, 0, 0}, 0, 0, 0, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, 0u};
  }
}
}  // namespace tx
