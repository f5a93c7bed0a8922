// rock.cuh -- rock tables (RockJfunc) evaluated on the device and on the host.
//
// Reference: RockJfunc::krw/kro/capPress/capPressDeriv/satFromCapPress
// (common/RockJfunc.hpp:63-141) and the per-cell dispatch of ReservoirPropertyCommon
// (common/ReservoirPropertyCommon_impl.hpp:466-528).  The tables are opm-core
// NonuniformTableLinear objects in the reference (that library is not part of the reference
// tree): here they are piecewise linear with the end value outside the table; the derivative is
// the slope of the interval holding the point (0 outside); the inverse of the J table
// interpolates s in J with the table read in increasing-J order (kept as a second copy, Jx/sy).
#pragma once

#include <cmath>

namespace porsol {

struct RockView {
    int nrock = 0;                 // 0: no tables (kr1 = s^2, kr2 = (1-s)^2, pc = 1e5 (1-s))
    const int* pos = nullptr;      // [nrock + 1] row range of each rock
    const double* s = nullptr;     // saturations, non-decreasing per rock
    const double* krw = nullptr;
    const double* kro = nullptr;
    const double* J = nullptr;
    const double* Jx = nullptr;    // J in increasing order ...
    const double* sy = nullptr;    // ... with the matching saturations
    const int* cell = nullptr;     // rock of each cell
    const double* skp = nullptr;   // per cell sqrt(tr K / (3 phi)) (J scaling)
    int jscale = 1;
    double sct = 1.0;              // sigma cos(theta)
};

// interval [lo, lo + 1] of x (non-decreasing, n >= 2) with x[lo] <= v < x[lo + 1], for
// x[0] < v < x[n - 1]
__host__ __device__ inline int tab_interval(const double* x, int n, double v)
{
    int lo = 0, hi = n - 1;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (x[mid] <= v) lo = mid;
        else hi = mid;
    }
    return lo;
}

__host__ __device__ inline double tab_value(const double* x, const double* y, int n, double v)
{
    if (v <= x[0]) return y[0];
    if (v >= x[n - 1]) return y[n - 1];
    const int lo = tab_interval(x, n, v);
    const double w = (v - x[lo]) / (x[lo + 1] - x[lo]);
    return (1.0 - w) * y[lo] + w * y[lo + 1];
}

__host__ __device__ inline double tab_slope(const double* x, const double* y, int n, double v)
{
    if (n < 2 || v < x[0] || v > x[n - 1]) return 0.0;
    const int lo = v >= x[n - 1] ? n - 2 : tab_interval(x, n, v);
    return x[lo + 1] > x[lo] ? (y[lo + 1] - y[lo]) / (x[lo + 1] - x[lo]) : 0.0;
}

// relative permeability of phase 0 (krw) or 1 (kro) in cell c
__host__ __device__ inline double rock_kr(const RockView& R, int phase, int c, double s)
{
    const int r = R.cell[c], a = R.pos[r], n = R.pos[r + 1] - a;
    return tab_value(R.s + a, (phase == 0 ? R.krw : R.kro) + a, n, s);
}

// RockJfunc::capPress
__host__ __device__ inline double rock_pc(const RockView& R, int c, double s)
{
    const int r = R.cell[c], a = R.pos[r], n = R.pos[r + 1] - a;
    const double j = tab_value(R.s + a, R.J + a, n, s);
    return R.jscale ? j * R.sct / R.skp[c] : j;
}

// RockJfunc::satFromCapPress: inverse J curve, clamped to [s_min, s_max] of the rock
__host__ __device__ inline double rock_sat(const RockView& R, int c, double pc)
{
    const int r = R.cell[c], a = R.pos[r], n = R.pos[r + 1] - a;
    const double v = R.jscale ? pc * R.skp[c] / R.sct : pc;
    const double s = tab_value(R.Jx + a, R.sy + a, n, v);
    return fmin(R.s[a + n - 1], fmax(R.s[a], s));
}

}  // namespace porsol
