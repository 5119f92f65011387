// Device-side continuum grid ("turi") and TTM state.
#pragma once

#include "fmdg.h"

#define FMDG_MAXT 4   // turies per system

struct TtmParams
{
    int type, ratio;
    unsigned min_atoms;
    int nC, nG;
    double C_gamma, K, G, dz2, frontsurf;
    double laser_t0, laser_tdiff, laser_m_2sig2_inv, laser_m_absdepth_inv, laser_factor;
    double Kzh_v2, Kzh_A, Kzh_B;
    const double *T_C, *Ct, *C_DD, *T_G, *Gt, *G_DD;   // device copies (type 2)
};

struct DTuri
{
    int dims[3];          // local dimensions including the turi margin
    int g2l[3];           // itc_local = itc_global + g2l
    int ncells;
    int itc_lo, itc_hi;   // interior range along z (1-D TTM)
    int ttm;              // 1 when a TTM solver is attached
    double tcellh[3], inv_tcellh[3], tcell_volume;
    double starttime, stoptime;
    long long *acc;       // 5 per cell, 64-bit fixed point: sum m, sum m v (3); count (integer)
    long long *tacc;      // sum m |v - vcm|^2, 64-bit fixed point
    double *mass, *vcm, *Ti;
    unsigned *num;
    double *Te, *Te2, *xi, *Ke, *Ce, *Gc, *srcz;
    double *Te_pre;       // Te after cell activation, before the substeps
    TtmParams p;
};
