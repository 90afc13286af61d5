// tables.cuh — the pair-operator packing shared by k_tables (setup.cu) and
// k_tables_tc (tables_tc.cu): the 18 direction-pair coefficients of one
// (outgoing o, incoming Gauss i) pair from the 13 phase-table products, and
// the 36 operator entries they give.
#pragma once
#include "common.cuh"

// The 18 coefficients (rt_sos_operator.c:54-72) from the sums over l of the 13
// products A_k = (incoming basis) x (outgoing basis x moment) of the pair:
// S[k] over all l, D[k] with the sign (-1)^(l+m), k in the numbering
//   0 P_i P_o beta    1 P_i R_o gamma   2 P_i T_o gamma   3 T_i T_o zeta
//   4 R_i R_o alpha   5 T_i R_o alpha   6 R_i T_o zeta    7 T_i T_o alpha
//   8 R_i R_o zeta    9 T_i P_o gamma  10 R_i P_o gamma  11 R_i T_o alpha
//  12 T_i R_o zeta
// (0..8: the table at [row i, column o]; 9..12: the transposed pair).  The
// value at column +o is S, at -o sigma D with sigma from the column basis.
__device__ inline void pair_coefs(const float *S, const float *D, float *c)
{
    c[0] = S[0];             c[1] = D[0];               // pfm[i][+-o]
    c[2] = S[2];             c[3] = -D[2];              // gt[i][+-o]
    c[4] = S[9];             c[5] = -D[9];              // gt[o][+-i]
    c[6] = S[1];             c[7] = D[1];               // gr[i][+-o]
    c[8] = S[10];            c[9] = D[10];              // gr[o][+-i]
    c[10] = S[3] + S[4];     c[11] = -D[3] + D[4];      // arr[i][+-o]
    c[12] = S[5] + S[6];     c[13] = D[5] - D[6];       // art[i][+-o]
    c[14] = S[11] + S[12];   c[15] = D[11] - D[12];     // art[o][+-i]
    c[16] = S[7] + S[8];     c[17] = -D[7] + D[8];      // att[i][+-o]
}

// The 36 operator entries of one (outgoing o, incoming Gauss i) pair from
// the 18 direction-pair coefficients of rt_sos_operator.c:54-72
// (order: ii_s ii_c iu_s iu_c iuT_s iuT_c iq_s iq_c iqT_s iqT_c qq_s qq_c
//  qu_s qu_c quT_s quT_c uu_s uu_c), with the quadrature weight folded in:
// st(ob, ib, v) for output block ob = 2 s_out + h_out and input block
// ib = 2 s_in + h_in.  The signs are those of the contraction in
// rt_sos_operator.c:387-406.
// The placement itself: st(ob, ib, q, neg) puts coefficient q (negated when
// neg) at output block ob, input block ib.
template <class Store>
__device__ inline void put_pair_places(Store st)
{
    enum { II_S, II_C, IU_S, IU_C, IUT_S, IUT_C, IQ_S, IQ_C, IQT_S, IQT_C, QQ_S, QQ_C,
           QU_S, QU_C, QUT_S, QUT_C, UU_S, UU_C };
    auto at = [&](int so, int ho, int si, int hi, int q, bool neg) { st(so * 2 + ho, si * 2 + hi, q, neg); };
    // I up / down
    at(0, 0, 0, 0, II_S, false);   at(0, 0, 1, 0, IQT_S, false);  at(0, 0, 2, 0, IUT_S, true);
    at(0, 0, 0, 1, II_C, false);   at(0, 0, 1, 1, IQT_C, false);  at(0, 0, 2, 1, IUT_C, true);
    at(0, 1, 0, 0, II_C, false);   at(0, 1, 1, 0, IQT_C, false);  at(0, 1, 2, 0, IUT_C, false);
    at(0, 1, 0, 1, II_S, false);   at(0, 1, 1, 1, IQT_S, false);  at(0, 1, 2, 1, IUT_S, false);
    // Q up / down
    at(1, 0, 0, 0, IQ_S, false);   at(1, 0, 1, 0, QQ_S, false);   at(1, 0, 2, 0, QU_S, true);
    at(1, 0, 0, 1, IQ_C, false);   at(1, 0, 1, 1, QQ_C, false);   at(1, 0, 2, 1, QU_C, false);
    at(1, 1, 0, 0, IQ_C, false);   at(1, 1, 1, 0, QQ_C, false);   at(1, 1, 2, 0, QU_C, true);
    at(1, 1, 0, 1, IQ_S, false);   at(1, 1, 1, 1, QQ_S, false);   at(1, 1, 2, 1, QU_S, false);
    // U up / down (leading minus of rt_sos_operator.c:399-406 folded in)
    at(2, 0, 0, 0, IU_S, true);    at(2, 0, 1, 0, QUT_S, true);   at(2, 0, 2, 0, UU_S, false);
    at(2, 0, 0, 1, IU_C, false);   at(2, 0, 1, 1, QUT_C, true);   at(2, 0, 2, 1, UU_C, false);
    at(2, 1, 0, 0, IU_C, true);    at(2, 1, 1, 0, QUT_C, false);  at(2, 1, 2, 0, UU_C, false);
    at(2, 1, 0, 1, IU_S, false);   at(2, 1, 1, 1, QUT_S, false);  at(2, 1, 2, 1, UU_S, false);
}

template <class Store>
__device__ inline void put_pair_blocks(Store st, float w, const float *c)
{
    put_pair_places([&](int ob, int ib, int q, bool neg) { st(ob, ib, neg ? -w * c[q] : w * c[q]); });
}

// The same entries at (operator row col_of(o), input column ib * N + i).
template <class Store>
__device__ inline void put_pair(Store st, const Geom &G, int o, int i, float w, const float *c)
{
    put_pair_blocks([&](int ob, int ib, float v) { st(col_of(G, ob >> 1, ob & 1, o), ib * G.N + i, v); }, w, c);
}
