/*
 * ORACLE — test infrastructure, not product code.
 *
 * A CPU restatement (C++17, FP64, OpenMP) of InterfaceAdvection.jl's per-step
 * hot path, written to follow the reference's loops, ranges, buffer aliasing
 * and operation order one to one.  Each function cites the reference lines it
 * restates (paths relative to the InterfaceAdvection.jl project root).
 *
 * WaterLily.jl (compat "1.8", not vendored, version unpinned) supplies BC!,
 * perBC!, accelerate!, ∂, ϕ, div, flux_out, median, mult and the Poisson
 * solver.  Those are restated here from their mathematical role as the
 * reference uses them, not from WaterLily's source.  The Poisson solve is the
 * reference's own in-repo Jacobi-PCG (src/flow.jl:300-326) with an L-infinity
 * stopping test; pressure is therefore pinned only by its FP64 residual.
 *
 * Pinning: the known-answer assertions of test/maintests.jl are transcribed in
 * tests/test_oracle_golden.py and run against this library.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py (cpu_baseline and the
 * `--impl reference` arm) load this library.
 */
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace {

struct G {
    int D, per;
    long n[3], s[3], N;
    explicit G(const orc_grid* g) : D(g->D), per(g->per) {
        for (int d = 0; d < 3; ++d) n[d] = g->n[d];
        if (D == 2) n[2] = 1;
        s[0] = 1; s[1] = n[0]; s[2] = n[0] * n[1];
        N = n[0] * n[1] * n[2];
    }
    bool isper(int d) const { return (per >> d) & 1; }
    void coords(long I, long c[3]) const {
        c[0] = I % n[0]; c[1] = (I / n[0]) % n[1]; c[2] = I / (n[0] * n[1]);
    }
    long lin(const long c[3]) const { return c[0] + s[1] * c[1] + s[2] * c[2]; }
};

/* Loop over the inclusive box lo..hi (third dimension collapsed in 2D). */
template <class F>
void box(const G& g, const long lo[3], const long hi[3], F&& fn) {
    long k0 = g.D == 3 ? lo[2] : 0, k1 = g.D == 3 ? hi[2] : 0;
#pragma omp parallel for collapse(2) schedule(static)
    for (long k = k0; k <= k1; ++k)
        for (long j = lo[1]; j <= hi[1]; ++j)
            for (long i = lo[0]; i <= hi[0]; ++i) {
                long c[3] = {i, j, k};
                fn(i + g.s[1] * j + g.s[2] * k, c);
            }
}
/* inside(f): 1..n-2 in every dimension */
template <class F>
void inside(const G& g, F&& fn) {
    long lo[3] = {1, 1, 1}, hi[3] = {g.n[0] - 2, g.n[1] - 2, g.n[2] - 2};
    box(g, lo, hi, fn);
}
/* every cell */
template <class F>
void allcells(const G& g, F&& fn) {
    long lo[3] = {0, 0, 0}, hi[3] = {g.n[0] - 1, g.n[1] - 1, g.n[2] - 1};
    box(g, lo, hi, fn);
}
/* WaterLily slice(N, i, j, low): index i along j, low..n-1 elsewhere */
template <class F>
void slice(const G& g, long i, int j, long low, F&& fn) {
    long lo[3], hi[3];
    for (int d = 0; d < 3; ++d) { lo[d] = low; hi[d] = g.n[d] - 1; }
    lo[j] = hi[j] = i;
    box(g, lo, hi, fn);
}
/* WaterLily inside_u(N, j): 2..n-2 along j, 1..n-1 elsewhere (0-based) */
template <class F>
void inside_u(const G& g, int j, F&& fn) {
    long lo[3], hi[3];
    for (int d = 0; d < 3; ++d) { lo[d] = 1; hi[d] = g.n[d] - 1; }
    lo[j] = 2; hi[j] = g.n[j] - 2;
    box(g, lo, hi, fn);
}
/* CIj(j, I, k): I with coordinate j replaced by k */
inline long cij(const G& g, int j, const long c[3], long k) {
    long cc[3] = {c[0], c[1], c[2]};
    cc[j] = k;
    return g.lin(cc);
}

inline double jsign(double x) { return x > 0 ? 1.0 : (x < 0 ? -1.0 : x); }

/* ===================== PLIC (src/PLIC.jl) ===================== */

template <class T> inline void sort2(T& a, T& b) { if (!(a < b)) std::swap(a, b); }  // :178
template <class T> inline void sort3(T& a, T& b, T& c) {                              // :186-191
    if (a > c) std::swap(a, c);
    if (a > b) std::swap(a, b);
    if (b > c) std::swap(b, c);
}
template <class T> inline T jmin(T a, T b) { return b < a ? b : a; }
template <class T> inline T jmax(T a, T b) { return a < b ? b : a; }

// α2f 2D, PLIC.jl:92
template <class T> T a2f(T m1, T m2, T a) { return a < m1 ? a * a / (2 * m1 * m2) : (a - m1 / 2) / m2; }
// α2f 3D, PLIC.jl:93-107
template <class T> T a2f(T m1, T m2, T m3, T a) {
    T m12 = m1 + m2;
    if (a < m1) return a * a * a / (6 * m1 * m2 * m3);
    if (a < m2) return a * (a - m1) / (2 * m2 * m3) + (m2 == 0 ? T(1) : m1 / m2) * m1 / (6 * m3);
    if (a < jmin(m3, m12))
        return (a * a * (3 * m12 - a) + m1 * m1 * (m1 - 3 * a) + m2 * m2 * (m2 - 3 * a)) / (6 * m1 * m2 * m3);
    if (m3 < m12)
        return (a * a * (3 - 2 * a) + m1 * m1 * (m1 - 3 * a) + m2 * m2 * (m2 - 3 * a) + m3 * m3 * (m3 - 3 * a)) /
               (6 * m1 * m2 * m3);
    return (2 * a - m12) / (2 * m3);
}
// proot, PLIC.jl:165-176
template <class T> T proot(T c0, T c1, T c2, T c3) {
    T a0 = c0 / c3, a1 = c1 / c3, a2 = c2 / c3;
    T p0 = a1 / 3 - a2 * a2 / 9;
    T q0 = (a1 * a2 - 3 * a0) / 6 - a2 * a2 * a2 / 27;
    T a = q0 / std::sqrt(-p0 * p0 * p0);
    T t = std::acos(a * a <= 1 ? a : T(0)) / 3;
    return std::sqrt(-p0) * (std::sqrt(T(3)) * std::sin(t) - std::cos(t)) - a2 / 3;
}
// f2α 2D, PLIC.jl:117
template <class T> T f2a(T m1, T m2, T v) { return v < m1 / (2 * m2) ? std::sqrt(2 * m1 * m2 * v) : m2 * v + m1 / 2; }
// f2α 3D, PLIC.jl:118-149
template <class T> T f2a(T m1, T m2, T m3, T v) {
    T m12 = m1 + m2;
    T p = 6 * m1 * m2 * m3;
    T v1 = (m2 == 0 ? T(1) : m1 / m2) * m1 / (6 * m3);
    T v2 = v1 + (m2 - m1) / (2 * m3);
    T v3 = m3 < m12 ? (m3 * m3 * (3 * m12 - m3) + m1 * m1 * (m1 - 3 * m3) + m2 * m2 * (m2 - 3 * m3)) / p
                    : m12 / (2 * m3);
    if (v < v1) return std::cbrt(p * v);
    if (v < v2) return (m1 + std::sqrt(m1 * m1 + 8 * m2 * m3 * (v - v1))) / 2;
    if (v < v3) return proot<T>(m1 * m1 * m1 + m2 * m2 * m2 - p * v, -3 * (m1 * m1 + m2 * m2), 3 * m12, T(-1));
    if (m3 < m12)
        return proot<T>(m1 * m1 * m1 + m2 * m2 * m2 + m3 * m3 * m3 - p * v, -3 * (m1 * m1 + m2 * m2 + m3 * m3),
                        T(3), T(-2));
    return m3 * v + m12 / 2;
}
// getIntercept 2D, PLIC.jl:20-29
template <class T> T get_intercept(T n1, T n2, T g) {
    T t = std::fabs(n1) + std::fabs(n2), a;
    if (g != T(0.5)) {
        T m1 = std::fabs(n1) / t, m2 = std::fabs(n2) / t;
        sort2(m1, m2);
        a = f2a(m1, m2, g < T(0.5) ? g : 1 - g);
    } else a = T(0.5);
    return (g < T(0.5) ? a : 1 - a) * t + jmin(n1, T(0)) + jmin(n2, T(0));
}
// getIntercept 3D, PLIC.jl:30-39
template <class T> T get_intercept(T n1, T n2, T n3, T g) {
    T t = std::fabs(n1) + std::fabs(n2) + std::fabs(n3), a;
    if (g != T(0.5)) {
        T m1 = std::fabs(n1) / t, m2 = std::fabs(n2) / t, m3 = std::fabs(n3) / t;
        sort3(m1, m2, m3);
        a = f2a(m1, m2, m3, g < T(0.5) ? g : 1 - g);
    } else a = T(0.5);
    return (g < T(0.5) ? a : 1 - a) * t + jmin(n1, T(0)) + jmin(n2, T(0)) + jmin(n3, T(0));
}
// getVolumeFraction 2D, PLIC.jl:59-70
template <class T> T get_vf(T n1, T n2, T b) {
    T t = std::fabs(n1) + std::fabs(n2);
    T a = (b - jmin(n1, T(0)) - jmin(n2, T(0))) / t;
    if (a <= 0 || a == T(0.5) || a >= 1) return jmin(jmax(a, T(0)), T(1));
    T m1 = std::fabs(n1) / t, m2 = std::fabs(n2) / t;
    sort2(m1, m2);
    T v = a2f(m1, m2, a < T(0.5) ? a : 1 - a);
    return a < T(0.5) ? v : 1 - v;
}
// getVolumeFraction 3D, PLIC.jl:71-82
template <class T> T get_vf(T n1, T n2, T n3, T b) {
    T t = std::fabs(n1) + std::fabs(n2) + std::fabs(n3);
    T a = (b - jmin(n1, T(0)) - jmin(n2, T(0)) - jmin(n3, T(0))) / t;
    if (a <= 0 || a == T(0.5) || a >= 1) return jmin(jmax(a, T(0)), T(1));
    T m1 = std::fabs(n1) / t, m2 = std::fabs(n2) / t, m3 = std::fabs(n3) / t;
    sort3(m1, m2, m3);
    T v = a2f(m1, m2, m3, a < T(0.5) ? a : 1 - a);
    return a < T(0.5) ? v : 1 - v;
}
inline double intercept_D(int D, const double n[3], double g) {
    return D == 2 ? get_intercept(n[0], n[1], g) : get_intercept(n[0], n[1], n[2], g);
}
inline double vf_D(int D, const double n[3], double b) {
    return D == 2 ? get_vf(n[0], n[1], b) : get_vf(n[0], n[1], n[2], b);
}

/* ===================== util / VOFutil ===================== */

// get3CellHeight, VOFutil.jl:158
inline double h3(const G& g, const double* f, long I, int s) { return f[I] + f[I - g.s[s]] + f[I + g.s[s]]; }
// fullorempty, VOFutil.jl:151 ; containInterface, VOFutil.jl:144
inline bool fullorempty(double x) { return x == 0 || x == 1; }
inline bool contain_interface(double x) { return 0 < x && x < 1; }
// myArgAbsMax, util.jl:19-31 (returns 0-based)
inline int argabsmax(int D, const double n[3]) {
    double mx = 0; int im = 0;
    for (int i = 0; i < D; ++i) {
        double c = n[i] * n[i];
        if (c > mx) { mx = c; im = i; }
    }
    return im;
}
// linInterpProp, VOFutil.jl:166
inline double lin_prop(double f, double lam) { return lam + (1 - lam) * f; }

/* ---- normal schemes (src/normalEstimation.jl); n is the cell's n̂[I,:] ---- */
// _PCD!, normalEstimation.jl:161-165
void nrm_pcd(const G& g, const double* f, long I, double n[3]) {
    for (int d = 0; d < g.D; ++d) n[d] = f[I - g.s[d]] - f[I + g.s[d]];
}
// _Column!, normalEstimation.jl:75-97
void nrm_column(const G& g, const double* f, long I, double n[3]) {
    nrm_pcd(g, f, I, n);
    int dom = argabsmax(g.D, n);
    for (int d = 0; d < g.D; ++d) {
        if (d == dom) { double sg = jsign(n[d]); n[d] = sg == 0 ? 1.0 : sg; continue; }
        double hl = h3(g, f, I - g.s[d], dom), hr = h3(g, f, I + g.s[d], dom);
        n[d] = (hl - hr) / 2;
    }
}
// _WY!, normalEstimation.jl:35-68
void nrm_wy(const G& g, const double* f, long I, double n[3]) {
    nrm_pcd(g, f, I, n);
    int dom = argabsmax(g.D, n);
    for (int d = 0; d < g.D; ++d) {
        if (d == dom) { double sg = jsign(n[d]); n[d] = sg == 0 ? 1.0 : sg; continue; }
        double hl = h3(g, f, I - g.s[d], dom), hc = h3(g, f, I, dom), hr = h3(g, f, I + g.s[d], dom);
        n[d] = (hl - hr) / 2;
        n[d] = std::fabs(n[d]) > 0.5 ? (n[d] * (hc - 1.5) >= 0.0 ? hc - hr : hl - hc) : n[d];
    }
}
// _WH!, normalEstimation.jl:105-154
void nrm_wh(const G& g, const double* f, long I, double n[3]) {
    nrm_column(g, f, I, n);
    int ad = argabsmax(g.D, n);                       // majorDir (util.jl:72-75)
    long dsg = std::signbit(n[ad]) ? -1 : 1;
    double an = std::fabs(n[ad]);
    an = an == 0 ? 1.0 : an;
    for (int d = 0; d < g.D; ++d) n[d] /= an;
    for (int d = 0; d < g.D; ++d) {
        if (d == ad) continue;
        double slope = std::fabs(n[d]);
        long csg = std::signbit(n[d]) ? -1 : 1;          // curDir = copysign(d, n̂[I,d])
        long off = csg * g.s[d];
        double hl = h3(g, f, I - off, ad), hc = h3(g, f, I, ad), hr = h3(g, f, I + off, ad);
        double sh = hl + hc + hr;
        if (4.5 * slope <= sh && sh <= 9 - 4.5 * slope) continue;
        double lim = jmin(1 / (2 * slope), 4.5 * slope);
        if (sh < 4.5 * slope) {
            double wb = h3(g, f, I - dsg * g.s[ad], d);
            if (wb > lim) n[d] = std::copysign((hl - 0.5) / (wb - 0.5), double(csg));
        }
        if (sh > 9 - 4.5 * slope) {
            double wt = h3(g, f, I + dsg * g.s[ad], d);
            if (wt < 3 - lim) n[d] = std::copysign((2.5 - hr) / (2.5 - wt), double(csg));
        }
    }
}
// _SLIC!, normalEstimation.jl:172-176
void nrm_slic(const G& g, const double* f, long I, double n[3]) {
    nrm_pcd(g, f, I, n);
    int dd = argabsmax(g.D, n);
    for (int i = 0; i < g.D; ++i) n[i] = i == dd ? jsign(n[i]) : 0.0;
}
// YoungSum, normalEstimation.jl:248-257 (CartesianIndices order: first dimension fastest)
double young_sum(const G& g, const double* f, long I, int d) {
    double a = 0;
    if (g.D == 2) {
        int e = 1 - d;
        for (int ii = -1; ii <= 0; ++ii)
            for (int iii = ii; iii <= ii + 1; ++iii) a += f[I + iii * g.s[e]];
    } else {
        int e0 = d == 0 ? 1 : 0, e1 = d == 2 ? 1 : 2;
        for (int i1 = -1; i1 <= 0; ++i1)
            for (int i0 = -1; i0 <= 0; ++i0)
                for (int j1 = i1; j1 <= i1 + 1; ++j1)
                    for (int j0 = i0; j0 <= i0 + 1; ++j0) a += f[I + j0 * g.s[e0] + j1 * g.s[e1]];
    }
    return a;
}
// _Y!, normalEstimation.jl:232-247
void nrm_y(const G& g, const double* f, long I, double n[3]) {
    double a = 0;
    for (int d = 0; d < g.D; ++d) {
        n[d] = (young_sum(g, f, I - g.s[d], d) - young_sum(g, f, I + g.s[d], d)) * 0.5;
        a += std::fabs(n[d]);
    }
    if (a == 0) for (int d = 0; d < g.D; ++d) n[d] = 1.0 / g.D;
    else for (int d = 0; d < g.D; ++d) n[d] /= a;
}
// _CCi, normalEstimation.jl:210-224
void nrm_cci(const G& g, const double* f, long I, int dc, const double n[3], double out[3]) {
    double s = 0;
    for (int d = 0; d < g.D; ++d) {
        if (d == dc) { double sg = jsign(n[d]); out[d] = sg == 0 ? 1.0 : sg; }
        else {
            double hu = h3(g, f, I + g.s[d], dc), hd = h3(g, f, I - g.s[d], dc);
            out[d] = -(hu - hd) / 2;
        }
        s += std::fabs(out[d]);
    }
    for (int d = 0; d < g.D; ++d) out[d] /= s;
}
// _MYC!, normalEstimation.jl:185-202
void nrm_myc(const G& g, const double* f, long I, double n[3]) {
    nrm_y(g, f, I, n);
    double mx = 0;
    for (int i = 0; i < g.D; ++i) mx = std::fabs(n[i]) > mx ? std::fabs(n[i]) : mx;
    double cur0 = 0; int cz = 0;
    double tmp[3];
    for (int iz = 0; iz < g.D; ++iz) {
        nrm_cci(g, f, I, iz, n, tmp);
        if (std::fabs(tmp[iz]) > cur0) cz = iz;
        cur0 = std::fabs(tmp[iz]);
    }
    nrm_cci(g, f, I, cz, n, tmp);
    if (std::fabs(tmp[cz]) < mx) for (int i = 0; i < g.D; ++i) n[i] = tmp[i];
}
// _CD! / crossSummation, normalEstimation.jl:266-277 (γ = 1)
double cross_sum(const G& g, const double* f, long I, int d) {
    double a = f[I];
    for (int e = 0; e < g.D; ++e) a += e != d ? (f[I - g.s[e]] + f[I + g.s[e]]) : 0.0;
    return a;
}
void nrm_cd(const G& g, const double* f, long I, double n[3]) {
    for (int d = 0; d < g.D; ++d) n[d] = (cross_sum(g, f, I - g.s[d], d) - cross_sum(g, f, I + g.s[d], d)) * 0.5;
}
// _XYLIC!, normalEstimation.jl:279-283 (default d = 2)
void nrm_xylic(const G& g, const double*, long, double n[3]) {
    for (int i = 0; i < g.D; ++i) n[i] = i == 1 ? 1.0 : 0.0;
}

bool normal(const G& g, int scheme, const double* f, long I, double n[3]) {
    n[0] = n[1] = n[2] = 0;
    switch (scheme) {
        case ORC_WH: nrm_wh(g, f, I, n); return true;
        case ORC_WY: nrm_wy(g, f, I, n); return true;
        case ORC_MYC: nrm_myc(g, f, I, n); return true;
        case ORC_Y: nrm_y(g, f, I, n); return true;
        case ORC_COLUMN: nrm_column(g, f, I, n); return true;
        case ORC_PCD: nrm_pcd(g, f, I, n); return true;
        case ORC_SLIC: nrm_slic(g, f, I, n); return true;
        case ORC_CD: nrm_cd(g, f, I, n); return true;
        case ORC_XYLIC: nrm_xylic(g, f, I, n); return true;
    }
    return false;
}

/* ---- boundary conditions ---- */
// BCf!, VOFutil.jl:64-75
void bcf(const G& g, double* f) {
    for (int j = 0; j < g.D; ++j) {
        long L = g.n[j] - 1;
        if (g.isper(j)) {
            slice(g, 0, j, 0, [&](long I, const long* c) { f[I] = f[cij(g, j, c, L - 1)]; });
            slice(g, L, j, 0, [&](long I, const long* c) { f[I] = f[cij(g, j, c, 1)]; });
        } else {
            slice(g, 0, j, 0, [&](long I, const long*) { f[I] = f[I + g.s[j]]; });
            slice(g, L, j, 0, [&](long I, const long*) { f[I] = f[I - g.s[j]]; });
        }
    }
}
// BCf!(d, f) VOFutil.jl:76-89 and BCv1D! VOFutil.jl:106-119 (identical rules)
void bcf_d(const G& g, int d, double* f) {
    for (int j = 0; j < g.D; ++j) {
        long L = g.n[j] - 1;
        if (g.isper(j)) {
            slice(g, 0, j, 0, [&](long I, const long* c) { f[I] = f[cij(g, j, c, L - 1)]; });
            slice(g, L, j, 0, [&](long I, const long* c) { f[I] = f[cij(g, j, c, 1)]; });
        } else if (j == d) {
            slice(g, 0, j, 0, [&](long I, const long*) { f[I] = f[I + 2 * g.s[j]]; });
        } else {
            slice(g, 0, j, 0, [&](long I, const long*) { f[I] = f[I + g.s[j]]; });
            slice(g, L, j, 0, [&](long I, const long*) { f[I] = f[I - g.s[j]]; });
        }
    }
}
// BCv!, VOFutil.jl:91-104
void bcv(const G& g, double* v) {
    for (int d = 0; d < g.D; ++d) bcf_d(g, d, v + d * g.N);
}
// BCVOF!, VOFutil.jl:44-62
void bcvof(const G& g, double* f, double* al, double* nh) {
    for (int j = 0; j < g.D; ++j) {
        long L = g.n[j] - 1;
        if (g.isper(j)) {
            auto cp = [&](long I, long S) {
                f[I] = f[S];
                for (int i = 0; i < g.D; ++i) nh[I + i * g.N] = nh[S + i * g.N];
                al[I] = al[S];
            };
            slice(g, 0, j, 0, [&](long I, const long* c) { cp(I, cij(g, j, c, L - 1)); });
            slice(g, L, j, 0, [&](long I, const long* c) { cp(I, cij(g, j, c, 1)); });
        } else {
            slice(g, 0, j, 0, [&](long I, const long*) { f[I] = f[I + g.s[j]]; });
            slice(g, L, j, 0, [&](long I, const long*) { f[I] = f[I - g.s[j]]; });
        }
    }
}
// WaterLily BC!(a, A, saveexit=false, perdir): normal component Dirichlet A[i] on the
// low ghost, the low wall face and the high wall face; tangential zero gradient;
// periodic wrap.  Loop order i (component) then j (dimension).
void bc_vel(const G& g, double* a, const double* A) {
    for (int i = 0; i < g.D; ++i) {
        double* ai = a + i * g.N;
        for (int j = 0; j < g.D; ++j) {
            long L = g.n[j] - 1;
            if (g.isper(j)) {
                slice(g, 0, j, 0, [&](long I, const long* c) { ai[I] = ai[cij(g, j, c, L - 1)]; });
                slice(g, L, j, 0, [&](long I, const long* c) { ai[I] = ai[cij(g, j, c, 1)]; });
            } else if (i == j) {
                for (long sidx : {0L, 1L}) slice(g, sidx, j, 0, [&](long I, const long*) { ai[I] = A[i]; });
                slice(g, L, j, 0, [&](long I, const long*) { ai[I] = A[i]; });
            } else {
                slice(g, 0, j, 0, [&](long I, const long*) { ai[I] = ai[I + g.s[j]]; });
                slice(g, L, j, 0, [&](long I, const long*) { ai[I] = ai[I - g.s[j]]; });
            }
        }
    }
}
// WaterLily perBC!(x, perdir): periodic wrap of a scalar on periodic dimensions only
void perbc(const G& g, double* x) {
    for (int j = 0; j < g.D; ++j) {
        if (!g.isper(j)) continue;
        long L = g.n[j] - 1;
        slice(g, 0, j, 0, [&](long I, const long* c) { x[I] = x[cij(g, j, c, L - 1)]; });
        slice(g, L, j, 0, [&](long I, const long* c) { x[I] = x[cij(g, j, c, 1)]; });
    }
}
// cleanWisp!, VOFutil.jl:127-136
void clean_wisp(const G& g, double* f, double tol) {
    inside(g, [&](long I, const long*) { f[I] = f[I] < tol ? 0.0 : (f[I] > 1 - tol ? 1.0 : f[I]); });
}
// WaterLily ϕ(d, I, f) = (f[I] + f[I-δd]) / 2
inline double phi(const G& g, int d, long I, const double* f) { return (f[I] + f[I - g.s[d]]) / 2; }
// f2face!, VOFutil.jl:229-234
void f2face(const G& g, double* ff, const double* f) {
    for (int d = 0; d < g.D; ++d) inside(g, [&](long I, const long*) { ff[I + d * g.N] = phi(g, d, I, f); });
    bcv(g, ff);
}
// getρ(d, I, f, λρ), VOFutil.jl:176
inline double rho_face(const G& g, int d, long I, const double* f, double lrho) { return lin_prop(phi(g, d, I, f), lrho); }
// getμ, VOFutil.jl:186-191
double getmu(const G& g, int i, int j, long I, const double* ff, double lmu, double mu, double lrho) {
    double f1 = ff[I - g.s[j] + i * g.N], f2 = ff[I + i * g.N], f3 = ff[I - g.s[i] + j * g.N], f4 = ff[I + j * g.N];
    double s = (f1 + f2 + f3 + f4) / 4;
    double fr = lrho < 1 ? jmin(jmin(f1, f2), jmin(f3, f4)) : jmax(jmax(f1, f2), jmax(f3, f4));
    return mu * jmin(lin_prop(s, lmu), (s > 0.5 ? 1.0 : lmu / lrho) * lin_prop(fr, lrho));
}

/* ===================== reconstruction + VOF advection ===================== */

// reconstructInterface!, normalEstimation.jl:10-28
void reconstruct(const G& g, int scheme, double* f, double* al, double* nh) {
    inside(g, [&](long I, const long*) {
        if (fullorempty(f[I])) {
            for (int i = 0; i < g.D; ++i) nh[I + i * g.N] = 0;
            al[I] = 0;
            return;
        }
        double n[3];
        normal(g, scheme, f, I, n);
        for (int i = 0; i < g.D; ++i) nh[I + i * g.N] = n[i];
        al[I] = intercept_D(g.D, n, f[I]);
    });
    bcvof(g, f, al, nh);
}

// getVOFFlux!, advection.jl:108-137 (fill!(fᶠ,0) then faces in inside_uWB(size(f),d))
void vof_flux(const G& g, double* fF, const double* f, const double* al, const double* nh, const double* u,
              const double* u0, double dt, int d, double* rhouf, double lrho) {
    std::fill(fF, fF + g.N, 0.0);
    long lo[3], hi[3];
    for (int e = 0; e < 3; ++e) { lo[e] = 1; hi[e] = g.n[e] - 2; }
    hi[d] = g.n[d] - 1;                                       // inside_uWB, util.jl:47-49
    box(g, lo, hi, [&](long IF, const long*) {
        double dl = dt / 2 * (u[IF + d * g.N] + u0[IF + d * g.N]);
        if (dl == 0) return;
        long IC = dl > 0 ? IF - g.s[d] : IF;
        double sa = 0;
        for (int ii = 0; ii < g.D; ++ii) sa += std::fabs(nh[IC + ii * g.N]);
        if (sa == 0 || fullorempty(f[IC])) {
            fF[IF] = f[IC] * dl;
        } else {
            double a = dl > 0 ? al[IC] - nh[IC + d * g.N] * (1 - dl) : al[IC];
            double nc[3] = {0, 0, 0};
            for (int ii = 0; ii < g.D; ++ii) nc[ii] = nh[IC + ii * g.N] * (ii == d ? std::fabs(dl) : 1.0);
            fF[IF] = vf_D(g.D, nc, a) * dl;
        }
        rhouf[IF + d * g.N] += dl * lrho + (1 - lrho) * fF[IF];   // fᶠ2ρuf, VOFutil.jl:218
    });
}

// WaterLily div(I, u) = Σ_d u[I+δd, d] - u[I, d]
inline double divu(const G& g, long I, const double* u) {
    double s = 0;
    for (int d = 0; d < g.D; ++d) s += u[I + g.s[d] + d * g.N] - u[I + d * g.N];
    return s;
}

// reportFillError, advection.jl:145-189 (findmax/findmin over the whole array)
void report_fill(const G& g, const double* f, const double* u, const double* u0, int d, double tol,
                 orc_fill_status* st) {
    double mx = -INFINITY, mn = INFINITY;
    long imx = 0, imn = 0;
    bool nan = false;
    for (long I = 0; I < g.N; ++I) {
        double v = f[I];
        if (v != v) { nan = true; continue; }
        if (v > mx) { mx = v; imx = I; }
        if (v < mn) { mn = v; imn = I; }
    }
    if (!st) return;
    if (nan) { st->nan = 1; st->dir = d; return; }
    auto interior = [&](long I) {
        long c[3]; g.coords(I, c);
        for (int e = 0; e < g.D; ++e) if (c[e] < 1 || c[e] > g.n[e] - 2) return false;
        return true;
    };
    if (mx - 1 > tol) {
        st->over = 1; st->maxf = mx; st->maxid = imx; st->dir = d;
        if (interior(imx)) {
            double du0 = std::fabs(divu(g, imx, u0)), du = std::fabs(divu(g, imx, u));
            if (du0 + du > 10 || du0 + du != du0 + du) st->diverge = 1;
        }
    }
    if (mn < -tol) {
        st->under = 1; st->minf = mn; st->minid = imn; st->dir = d;
        if (interior(imn)) {
            double du0 = std::fabs(divu(g, imn, u0)), du = std::fabs(divu(g, imn, u));
            if (du0 + du > 10 || du0 + du != du0 + du) st->diverge = 1;
        }
    }
}

// advectVOF1d!, advection.jl:80-89 (also the loop body of advectVOF!, advection.jl:60-73)
void advect_vof_1d(const G& g, int scheme, double* f, double* fF, double* al, double* nh, const double* u,
                   const double* u0, double dt, const int8_t* cbar, double* rhouf, double lrho, int d, double tol_rep,
                   double tol, orc_fill_status* st) {
    reconstruct(g, scheme, f, al, nh);
    vof_flux(g, fF, f, al, nh, u, u0, dt, d, rhouf, lrho);
    inside(g, [&](long I, const long*) {
        double du = u[I + g.s[d] + d * g.N] - u[I + d * g.N];
        double du0 = u0[I + g.s[d] + d * g.N] - u0[I + d * g.N];
        f[I] += fF[I] - fF[I + g.s[d]] + double(cbar[I]) * (du + du0) * dt / 2;
    });
    report_fill(g, f, u, u0, d, tol_rep, st);
    clean_wisp(g, f, tol);
    bcf(g, f);
}

/* ===================== momentum (src/flow.jl) ===================== */

// WaterLily median(a,b,c)
inline double median3(double a, double b, double c) { return jmax(jmin(a, b), jmin(jmax(a, b), c)); }
// limiters, flow.jl:5-15
double limiter(int which, double u, double c, double d) {
    switch (which) {
        case ORC_UPWIND: return c;
        case ORC_MINMOD: return median3((3 * c - u) / 2, c, (c + d) / 2);
        case ORC_KOREN: return median3((7 * c + d - 2 * u) / 6, c, median3(2 * c - u, c, d));
        case ORC_VANALBADA1: {
            double al = c - u, be = d - c;
            return c + jmax(al * be, 0.0) * ((al == be && al == 0) ? 0.0 : (al + be) / (al * al + be * be)) / 2;
        }
        case ORC_SWEBY:
        case ORC_SUPERBEE: {
            double gam = which == ORC_SWEBY ? 1.5 : 2.0;
            double s = jsign(d - u);
            if (c <= jmin(u, d) || c >= jmax(u, d)) return c;
            return c + s * jmax(jmax(0.0, jmin(s * gam * (c - u), s * (d - c))), jmin(s * (c - u), s * gam * (d - c))) / 2;
        }
        case ORC_TVDCEN: {
            double s = jsign(d - u);
            if (c <= jmin(u, d) || c >= jmax(u, d)) return c;
            return c + s * jmin(s * (c - u), s * (d - c) / 2);
        }
        case ORC_TVDDOWN: {
            double s = jsign(d - u);
            if (c <= jmin(u, d) || c >= jmax(u, d)) return c;
            return c + s * jmin(s * (c - u), s * (d - c));
        }
    }
    return c;
}

struct MomCtx {
    const G& g;
    const double *rhouf, *uStar, *fOld;
    double dt, lrho;
    int lim;
};
// Ψ = ϕ(i, CI(I,j), ρuf) = (ρuf[I,j] + ρuf[I-δi,j]) / 2
inline double psi_face(const MomCtx& m, int i, int j, long I) {
    return (m.rhouf[I + j * m.g.N] + m.rhouf[I - m.g.s[i] + j * m.g.N]) / 2;
}
// ϕq, flow.jl:37-57 (fOld is the face-averaged old fraction dρ)
double phiq(const MomCtx& m, int j, int i, long I, double uu, double cc, double dd) {
    double Psi = psi_face(m, i, j, I);
    long IC = Psi > 0 ? I - m.g.s[j] : I;
    double vI = cc, vd = limiter(m.lim, uu, cc, dd), va = 2 * vI - vd;
    double mOut = std::fabs(Psi) * m.dt;
    double mOld = lin_prop(m.fOld[IC + i * m.g.N], m.lrho);   // getρ(IiCell,fOld,λρ), VOFutil.jl:174
    if (mOut > mOld) return Psi * vI;
    double l2 = std::fabs(mOut) / mOld, l1 = 1 - l2;
    double vb = l2 * va + l1 * vd;
    return Psi * (vb + vd) / 2;
}
// ϕu / ϕuL / ϕuR / ϕuP, flow.jl:20-35 ; f = uStar component i
double phiu(const MomCtx& m, int j, int i, long I, double Psi) {
    const double* f = m.uStar + i * m.g.N;
    long s = m.g.s[j];
    return Psi > 0 ? phiq(m, j, i, I, f[I - 2 * s], f[I - s], f[I]) : phiq(m, j, i, I, f[I + s], f[I], f[I - s]);
}
double phiuL(const MomCtx& m, int j, int i, long I, double Psi) {
    const double* f = m.uStar + i * m.g.N;
    long s = m.g.s[j];
    return Psi > 0 ? phiq(m, j, i, I, 2 * f[I - s] - f[I], f[I - s], f[I]) : phiq(m, j, i, I, f[I + s], f[I], f[I - s]);
}
double phiuR(const MomCtx& m, int j, int i, long I, double Psi) {
    const double* f = m.uStar + i * m.g.N;
    long s = m.g.s[j];
    return Psi < 0 ? phiq(m, j, i, I, 2 * f[I] - f[I - s], f[I], f[I - s]) : phiq(m, j, i, I, f[I - 2 * s], f[I - s], f[I]);
}
double phiuP(const MomCtx& m, int j, int i, long Ip, long I, double Psi) {
    const double* f = m.uStar + i * m.g.N;
    long s = m.g.s[j];
    return Psi > 0 ? phiq(m, j, i, I, f[Ip], f[I - s], f[I]) : phiq(m, j, i, I, f[I + s], f[I], f[I - s]);
}

// advectρuu1D!, flow.jl:212-241
void advect_rhouu_1d(const G& g, double* rhou, double* r, double* Phi, const double* rhouf, const double* uStar,
                     const double* uOld, const double* fOld, double* dila, const double* u, const double* u0,
                     const int8_t* cbar, double lrho, int lim, int d, double dt) {
    std::fill(r, r + g.D * g.N, 0.0);
    int j = d;
    inside(g, [&](long I, const long*) {
        double dU = u[I + g.s[d] + d * g.N] - u[I + d * g.N], dU0 = u0[I + g.s[d] + d * g.N] - u0[I + d * g.N];
        dila[I] = lin_prop(double(cbar[I]), lrho) * (dU + dU0) / 2;
    });
    bcf(g, dila);
    MomCtx m{g, rhouf, uStar, fOld, dt, lrho, lim};
    long L = g.n[j] - 1;
    for (int i = 0; i < g.D; ++i) {
        double* ri = r + i * g.N;
        if (!g.isper(j)) {
            slice(g, 1, j, 1, [&](long I, const long*) { ri[I] += phiuL(m, j, i, I, psi_face(m, i, j, I)); });
        } else {
            slice(g, 1, j, 1, [&](long I, const long* c) {
                Phi[I] = phiuP(m, j, i, cij(g, j, c, L - 2), I, psi_face(m, i, j, I));
                ri[I] += Phi[I];
            });
        }
        inside_u(g, j, [&](long I, const long*) {
            Phi[I] = phiu(m, j, i, I, psi_face(m, i, j, I));
            ri[I] += Phi[I];
        });
        inside_u(g, j, [&](long I, const long*) { ri[I - g.s[j]] -= Phi[I]; });
        if (!g.isper(j)) {
            slice(g, L, j, 1, [&](long I, const long*) { ri[I - g.s[j]] += -phiuR(m, j, i, I, psi_face(m, i, j, I)); });
        } else {
            slice(g, L, j, 1, [&](long I, const long* c) { ri[I - g.s[j]] -= Phi[cij(g, j, c, 1)]; });
        }
        inside(g, [&](long I, const long*) { ri[I] += uOld[I + i * g.N] * phi(g, i, I, dila); });
    }
    for (long k = 0; k < g.D * g.N; ++k) rhou[k] += dt * r[k];      // axpy!(δt, r, ρu)
}

// ρu2u! / u2ρu!, VOFutil.jl:198-211
void rhou2u(const G& g, double* u, const double* rhou, const double* f, double lrho) {
    inside(g, [&](long I, const long*) {
        for (int d = 0; d < g.D; ++d) u[I + d * g.N] = rhou[I + d * g.N] / rho_face(g, d, I, f, lrho);
    });
}
void u2rhou(const G& g, double* rhou, const double* u, const double* f, double lrho) {
    inside(g, [&](long I, const long*) {
        for (int d = 0; d < g.D; ++d) rhou[I + d * g.N] = u[I + d * g.N] * rho_face(g, d, I, f, lrho);
    });
}

// advectVOFρuu!, flow.jl:165-210 with the aliasing of advectfq! (flow.jl:157-164):
// r = flow.f, Φ = flow.σ, uStar = intf.n̂, ρ̄∂ⱼuⱼ = intf.α, fOld = intf.dρ
void advect_vof_rhouu(const G& g, orc_state* s, double* f, const double* u1, const double* u2, const double* uOld,
                      double dt, const int* dirO, orc_fill_status* st) {
    const double tol = 10 * 2.220446049250313e-16;
    allcells(g, [&](long I, const long*) { s->cbar[I] = f[I] < 0.5 ? 0 : 1; });
    double* r = s->force;
    double* Phi = s->sigma;
    for (int k = 0; k < g.D; ++k) {
        int d = dirO[k];
        rhou2u(g, r, s->rhou, f, s->lrho);
        bc_vel(g, r, s->uBC);
        std::memcpy(Phi, f, sizeof(double) * g.N);
        std::fill(s->rhouf, s->rhouf + g.D * g.N, 0.0);
        advect_vof_1d(g, s->scheme, f, s->fF, s->alpha, s->nhat, u1, u2, dt, s->cbar, s->rhouf, s->lrho, d, 10 * tol,
                      tol, st);
        f2face(g, s->drho, Phi);
        std::memcpy(s->nhat, r, sizeof(double) * g.D * g.N);
        for (long q = 0; q < g.D * g.N; ++q) s->rhouf[q] *= 1 / dt;
        bc_vel(g, s->rhouf, s->uBC);
        advect_rhouu_1d(g, s->rhou, r, Phi, s->rhouf, s->nhat, uOld, s->drho, s->alpha, u1, u2, s->cbar, s->lrho,
                        s->limiter, d, dt);
    }
}

// viscF, flow.jl:144 ; ∂(j,CI(I,i),u) = u[I,i]-u[I-δj,i]
inline double viscF(const G& g, int i, int j, long I, const double* u, const double* ff, double lmu, double mu,
                    double lrho) {
    double dji = u[I + i * g.N] - u[I - g.s[j] + i * g.N];
    double dij = u[I + j * g.N] - u[I - g.s[i] + j * g.N];
    return getmu(g, i, j, I, ff, lmu, mu, lrho) * (dji + dij);
}
// visc!, flow.jl:119-153 (fFace = intf.n̂, Φ = flow.σ)
void visc(const G& g, double* r, const double* u, double* ff, double* Phi, const double* f, double lmu, double mu,
          double lrho) {
    f2face(g, ff, f);
    for (int i = 0; i < g.D; ++i)
        for (int j = 0; j < g.D; ++j) {
            double* ri = r + i * g.N;
            long L = g.n[j] - 1;
            if (!g.isper(j)) {
                slice(g, 1, j, 1, [&](long I, const long*) { ri[I] += -viscF(g, i, j, I, u, ff, lmu, mu, lrho); });
            } else {
                slice(g, 1, j, 1, [&](long I, const long*) {
                    Phi[I] = -viscF(g, i, j, I, u, ff, lmu, mu, lrho);
                    ri[I] += Phi[I];
                });
            }
            inside_u(g, j, [&](long I, const long*) {
                Phi[I] = -viscF(g, i, j, I, u, ff, lmu, mu, lrho);
                ri[I] += Phi[I];
            });
            inside_u(g, j, [&](long I, const long*) { ri[I - g.s[j]] -= Phi[I]; });
            if (!g.isper(j)) {
                slice(g, L, j, 1, [&](long I, const long*) { ri[I - g.s[j]] += viscF(g, i, j, I, u, ff, lmu, mu, lrho); });
            } else {
                slice(g, L, j, 1, [&](long I, const long* c) { ri[I - g.s[j]] -= Phi[cij(g, j, c, 1)]; });
            }
        }
}

/* ---- surface tension (src/surfaceTension.jl) ---- */
inline bool valid_ci(const G& g, const long c[3]) {
    for (int e = 0; e < g.D; ++e) if (c[e] < 0 || c[e] > g.n[e] - 1) return false;
    return true;
}
// getPopinetHeightAdaptive (monotonic), surfaceTension.jl:78-101 ; is = signed 1-based direction
double popinet_height(const G& g, const double* f, long I, int is) {
    int ax = std::abs(is) - 1;
    long sg = is > 0 ? 1 : -1;
    long c0[3]; g.coords(I, c0);
    long c[3] = {c0[0], c0[1], c0[2]};
    double fnow = f[I], H = fnow - 0.5;
    bool fin = fnow < 1;
    while (!fin || contain_interface(fnow)) {
        c[ax] += sg;
        if (!valid_ci(g, c)) break;
        double fv = f[g.lin(c)];
        fnow = fv > fnow ? 0.0 : fv;
        H += fnow;
        fin = contain_interface(fnow) ? true : fin;
    }
    c[0] = c0[0]; c[1] = c0[1]; c[2] = c0[2];
    fnow = f[I];
    fin = fnow > 0;
    while (!fin || contain_interface(fnow)) {
        c[ax] -= sg;
        if (!valid_ci(g, c)) break;
        double fv = f[g.lin(c)];
        fnow = fv < fnow ? 1.0 : fv;
        H += fnow - 1;
        fin = contain_interface(fnow) ? true : fin;
    }
    return H;
}
// getXdir / getXYdir, util.jl:64-65 (signed 1-based directions)
inline int sgnI(int i) { return i > 0 ? 1 : (i < 0 ? -1 : 0); }
inline int get_xdir(int i) { return std::abs(i) == 1 ? -2 * sgnI(i) : sgnI(i); }
inline void get_xydir(int i, int& ix, int& iy) {
    ix = sgnI(i) * ((std::abs(i)) % 3 + 1);
    iy = (std::abs(i) + 1) % 3 + 1;
}
// offset of δd(i, I) for a signed 1-based direction
inline long doff(const G& g, int i) { return i == 0 ? 0 : sgnI(i) * g.s[std::abs(i) - 1]; }
inline double root1p5(double a) { return std::sqrt(a * a * a); }
// getCurvature 3D / 2D, surfaceTension.jl:29-59
double curvature(const G& g, const double* f, long I, int i) {
    if (g.D == 3) {
        const double filt = 0.2;
        int ix, iy;
        get_xydir(i, ix, iy);
        double H[3][3];
        for (int yu = -1; yu <= 1; ++yu)
            for (int xu = -1; xu <= 1; ++xu)
                H[xu + 1][yu + 1] = popinet_height(g, f, I + xu * doff(g, ix) + yu * doff(g, iy), i);
        // Julia H[a,b] 1-based -> H[a-1][b-1]
        double Hx = (H[2][1] - H[0][1]) / 2, Hy = (H[1][2] - H[1][0]) / 2;
        double Hxx = ((H[2][1] + H[0][1] - 2 * H[1][1]) + (H[2][0] + H[0][0] - 2 * H[1][0]) * filt +
                      (H[2][2] + H[0][2] - 2 * H[1][2]) * filt) / (1 + 2 * filt);
        double Hyy = ((H[1][2] + H[1][0] - 2 * H[1][1]) + (H[0][2] + H[0][0] - 2 * H[0][1]) * filt +
                      (H[2][2] + H[2][0] - 2 * H[2][1]) * filt) / (1 + 2 * filt);
        double Hxy = (H[2][2] + H[0][0] - H[2][0] - H[0][2]) / 4;
        return (Hxx * (1 + Hy * Hy) + Hyy * (1 + Hx * Hx) - 2 * Hxy * Hx * Hy) / root1p5(1 + Hx * Hx + Hy * Hy);
    }
    int ix = get_xdir(i);
    double H[3];
    for (int xu = -1; xu <= 1; ++xu) H[xu + 1] = popinet_height(g, f, I + xu * doff(g, ix), i);
    double Hx = (H[2] - H[0]) / 2, Hxx = (H[2] + H[0] - 2 * H[1]);
    return Hxx / root1p5(1 + Hx * Hx);
}
// surfTen!, surfaceTension.jl:8-20 (fbuffer = intf.fᶠ, n̂ = intf.n̂)
void surften(const G& g, double* forcing, const double* f, double* nh, double* fb, double eta) {
    for (int d = 0; d < g.D; ++d) {
        inside(g, [&](long I, const long*) { fb[I] = phi(g, d, I, f); });
        bcf_d(g, d, fb);
        inside(g, [&](long I, const long*) {
            if (!contain_interface(fb[I])) return;
            double n[3] = {0, 0, 0};
            nrm_wy(g, fb, I, n);
            for (int e = 0; e < g.D; ++e) nh[I + e * g.N] = n[e];
        });
        inside(g, [&](long I, const long*) {
            if (!contain_interface(fb[I])) return;
            double n[3] = {0, 0, 0};
            for (int e = 0; e < g.D; ++e) n[e] = nh[I + e * g.N];
            int ia = argabsmax(g.D, n);
            int md = std::signbit(n[ia]) ? -(ia + 1) : (ia + 1);    // majorDir
            forcing[I + d * g.N] += eta * curvature(g, fb, I, md) * -(f[I] - f[I - g.s[d]]);
        });
    }
}

// updateU!, flow.jl:244-252 (constant gravity for accelerate!)
void update_u(const G& g, orc_state* s, double* u, double* rhou, const double* rhou0, double* forcing, double dt,
              const double* f, double w) {
    double a = 1 / w - 1;
    for (long k = 0; k < g.D * g.N; ++k) rhou[k] = (a * rhou0[k] + rhou[k] + forcing[k] * dt) * w;
    rhou2u(g, u, rhou, f, s->lrho);
    std::fill(forcing, forcing + g.D * g.N, 0.0);
    if (s->has_g)
        for (int i = 0; i < g.D; ++i)
            for (long k = 0; k < g.N; ++k) forcing[k + i * g.N] += s->g[i];
    for (long k = 0; k < g.D * g.N; ++k) u[k] += dt * w * forcing[k];
}
// updateL!, flow.jl:254-259
void update_L(const G& g, orc_state* s, const double* f) {
    for (int d = 0; d < g.D; ++d)
        inside(g, [&](long I, const long*) { s->mu0[I + d * g.N] /= rho_face(g, d, I, f, s->lrho); });
    double z[3] = {0, 0, 0};
    bc_vel(g, s->mu0, z);
}

/* ---- Poisson: WaterLily operator + the reference's Jacobi-PCG (flow.jl:300-326) ---- */
// diagonal D = -Σ (L[I,i] + L[I+δi,i]), iD = 1/D (0 when |D| tiny)
void set_diag(const G& g, orc_state* s) {
    const double* L = s->mu0;
    std::fill(s->pD, s->pD + g.N, 0.0);
    std::fill(s->piD, s->piD + g.N, 0.0);
    inside(g, [&](long I, const long*) {
        double dd = 0;
        for (int i = 0; i < g.D; ++i) dd -= L[I + i * g.N] + L[I + g.s[i] + i * g.N];
        s->pD[I] = dd;
        s->piD[I] = dd * dd < 2 * 2.220446049250313e-16 ? 0.0 : 1 / dd;
    });
}
inline double mult(const G& g, long I, const double* L, const double* Dg, const double* x) {
    double a = Dg[I] * x[I];
    for (int i = 0; i < g.D; ++i) a += x[I - g.s[i]] * L[I + i * g.N] + x[I + g.s[i]] * L[I + g.s[i] + i * g.N];
    return a;
}
double linf_inside(const G& g, const double* r) {
    double m = 0;
    long lo[3] = {1, 1, 1}, hi[3] = {g.n[0] - 2, g.n[1] - 2, g.n[2] - 2};
    if (g.D == 2) lo[2] = hi[2] = 0;
    for (long k = lo[2]; k <= hi[2]; ++k)
        for (long j = lo[1]; j <= hi[1]; ++j)
            for (long i = lo[0]; i <= hi[0]; ++i) m = jmax(m, std::fabs(r[i + g.s[1] * j + g.s[2] * k]));
    return m;
}
double dot_inside(const G& g, const double* a, const double* b) {
    double acc = 0;
    long lo[3] = {1, 1, 1}, hi[3] = {g.n[0] - 2, g.n[1] - 2, g.n[2] - 2};
    if (g.D == 2) lo[2] = hi[2] = 0;
#pragma omp parallel for collapse(2) reduction(+ : acc)
    for (long k = lo[2]; k <= hi[2]; ++k)
        for (long j = lo[1]; j <= hi[1]; ++j)
            for (long i = lo[0]; i <= hi[0]; ++i) {
                long I = i + g.s[1] * j + g.s[2] * k;
                acc += a[I] * b[I];
            }
    return acc;
}
void poisson_jacobi_pcg(const G& g, orc_state* s) {
    double *x = s->p, *r = s->pr, *e = s->peps, *z = s->pz, *L = s->mu0;
    std::vector<double> q(g.N, 0.0);
    set_diag(g, s);
    perbc(g, x);
    inside(g, [&](long I, const long*) { r[I] = s->sigma[I] - mult(g, I, L, s->pD, x); });
    double res = linf_inside(g, r);
    int it = 0;
    inside(g, [&](long I, const long*) { z[I] = e[I] = r[I] * s->piD[I]; });
    double rho = dot_inside(g, r, z);
    while (res > s->ptol && it < s->pitmx) {
        perbc(g, e);
        inside(g, [&](long I, const long*) { q[I] = mult(g, I, L, s->pD, e); });
        double alpha = rho / dot_inside(g, q.data(), e);
        inside(g, [&](long I, const long*) {
            x[I] += alpha * e[I];
            r[I] -= alpha * q[I];
        });
        inside(g, [&](long I, const long*) { z[I] = r[I] * s->piD[I]; });
        double rho2 = dot_inside(g, r, z);
        double beta = rho2 / rho;
        inside(g, [&](long I, const long*) { e[I] = beta * e[I] + z[I]; });
        rho = rho2;
        res = linf_inside(g, r);
        ++it;
    }
    perbc(g, x);
    s->piters = it;
    s->presid = res;
}
/* ---- Multigrid-preconditioned flexible CG: the solver the reference's default call site uses,
 * inproject!(…, ::MultiLevelPoisson) → WaterLily solver! (flow.jl:343-347).  WaterLily's source is not
 * available, so this is a geometric multigrid restated from the mathematics of the operator above, not
 * from WaterLily's code: cell-centred levels (2x coarsening while every interior extent is even and
 * >= 4), coarse face coefficient = ½ Σ of the 2^(D-1) fine faces it covers, restriction by the sum of
 * the 2^D children, prolongation by injection, symmetric red-black Gauss-Seidel (nu1 red→black sweeps
 * before, nu2 black→red after), the coarsest level swept from zero on its mean-free right-hand side.
 * The V-cycle preconditions a Polak–Ribière flexible CG that stops on the L∞ norm of the true residual
 * (the same test as the Jacobi-PCG above).  Only the converged pressure is compared (up to its free
 * constant), so the solver's internals need not match the product's. */
struct MGLevel {
    orc_grid og;
    G g;
    std::vector<double> Lown, Dg, x, b, r;
    const double* L = nullptr;
    explicit MGLevel(const orc_grid& o) : og(o), g(&og) {}
};
struct MGCache {
    long key[4] = {0, 0, 0, 0};
    std::vector<MGLevel> lv;
    std::vector<double> r, rold, sv, p, q;
};
static MGCache g_mg;

// neighbour offsets of interior cell I (coords c) along i, periodic ends wrapped
inline void nbr(const G& g, int i, long I, const long c[3], long& lo, long& hi) {
    lo = I - g.s[i];
    hi = I + g.s[i];
    if (g.isper(i)) {
        if (c[i] == 1) lo = I + (g.n[i] - 3) * g.s[i];
        if (c[i] == g.n[i] - 2) hi = I - (g.n[i] - 3) * g.s[i];
    }
}
inline double mg_off(const MGLevel& l, long I, const long c[3], const double* x) {
    const G& g = l.g;
    double a = 0;
    for (int i = 0; i < g.D; ++i) {
        long lo, hi;
        nbr(g, i, I, c, lo, hi);
        a += l.L[I + i * g.N] * x[lo] + l.L[I + g.s[i] + i * g.N] * x[hi];
    }
    return a;
}
void mg_rbgs(MGLevel& l, int color) {
    const G& g = l.g;
    inside(g, [&](long I, const long* c) {
        if (((c[0] + c[1] + c[2]) & 1) != color) return;
        if (l.Dg[I] == 0) return;
        l.x[I] = (l.b[I] - mg_off(l, I, c, l.x.data())) / l.Dg[I];
    });
}
void mg_build(const G& gf, const double* Lf) {
    const long key[4] = {gf.D, gf.per, gf.n[0] * 100003 + gf.n[1], gf.n[2]};
    bool same = g_mg.lv.size() && std::equal(key, key + 4, g_mg.key);
    if (!same) {
        g_mg.lv.clear();
        std::copy(key, key + 4, g_mg.key);
        orc_grid o{gf.D, gf.per, {gf.n[0], gf.n[1], gf.D == 3 ? gf.n[2] : 1}};
        g_mg.lv.reserve(32);
        g_mg.lv.emplace_back(o);
        while (true) {
            const orc_grid& c = g_mg.lv.back().og;
            bool ok = true;
            for (int d = 0; d < c.D; ++d) {
                long ni = c.n[d] - 2;
                if (ni % 2 != 0 || ni < 4) ok = false;
            }
            if (!ok) break;
            orc_grid o2{c.D, c.per, {(c.n[0] - 2) / 2 + 2, (c.n[1] - 2) / 2 + 2, c.D == 3 ? (c.n[2] - 2) / 2 + 2 : 1}};
            g_mg.lv.emplace_back(o2);
        }
        for (size_t k = 0; k < g_mg.lv.size(); ++k) {
            MGLevel& l = g_mg.lv[k];
            const long N = l.g.N;
            if (k > 0) l.Lown.assign(N * l.g.D, 0.0);
            l.Dg.assign(N, 0.0);
            l.x.assign(N, 0.0);
            l.b.assign(N, 0.0);
            l.r.assign(N, 0.0);
        }
        for (auto* v : {&g_mg.r, &g_mg.rold, &g_mg.sv, &g_mg.p, &g_mg.q}) v->assign(gf.N, 0.0);
    }
    g_mg.lv[0].L = Lf;
    for (size_t k = 1; k < g_mg.lv.size(); ++k) {
        MGLevel& l = g_mg.lv[k];
        const MGLevel& f = g_mg.lv[k - 1];
        const G& gc = l.g;
        const G& gg = f.g;
        double* Lc = l.Lown.data();
        for (int i = 0; i < gc.D; ++i) {
            // every coarse face 1..n-1 along i, interior elsewhere
            long lo[3] = {1, 1, 1}, hi[3] = {gc.n[0] - 2, gc.n[1] - 2, gc.n[2] - 2};
            hi[i] = gc.n[i] - 1;
            box(gc, lo, hi, [&](long Ic, const long* c) {
                long fb[3] = {2 * c[0] - 1, 2 * c[1] - 1, gc.D == 3 ? 2 * c[2] - 1 : 0};
                double acc = 0;
                const int o1 = i == 0 ? 1 : 0, o2 = i == 2 ? 1 : 2;
                for (int a = 0; a < 2; ++a)
                    for (int b2 = 0; b2 < (gc.D == 3 ? 2 : 1); ++b2) {
                        long ff[3] = {fb[0], fb[1], fb[2]};
                        ff[o1] += a;
                        if (gc.D == 3) ff[o2] += b2;
                        acc += f.L[gg.lin(ff) + i * gg.N];
                    }
                Lc[Ic + i * gc.N] = 0.5 * acc;
            });
        }
        l.L = Lc;
    }
    for (auto& l : g_mg.lv) {
        const G& g = l.g;
        inside(g, [&](long I, const long*) {
            double dd = 0;
            for (int i = 0; i < g.D; ++i) dd -= l.L[I + i * g.N] + l.L[I + g.s[i] + i * g.N];
            l.Dg[I] = dd;
        });
    }
}
void mg_vcycle(size_t k, int nu1, int nu2, int nuc) {
    MGLevel& l = g_mg.lv[k];
    const G& g = l.g;
    std::fill(l.x.begin(), l.x.end(), 0.0);
    if (k + 1 == g_mg.lv.size()) {
        double m = 0;
        long cnt = 0;
        for (long I = 0; I < g.N; ++I) {
            long c[3];
            g.coords(I, c);
            bool in = true;
            for (int e = 0; e < g.D; ++e) if (c[e] < 1 || c[e] > g.n[e] - 2) in = false;
            if (in) { m += l.b[I]; ++cnt; }
        }
        m /= double(cnt);
        inside(g, [&](long I, const long*) { l.b[I] -= m; });
        for (int it = 0; it < nuc; ++it) {
            mg_rbgs(l, 0); mg_rbgs(l, 1);
            mg_rbgs(l, 1); mg_rbgs(l, 0);
        }
        return;
    }
    for (int it = 0; it < nu1; ++it) { mg_rbgs(l, 0); mg_rbgs(l, 1); }
    inside(g, [&](long I, const long* c) { l.r[I] = l.b[I] - (l.Dg[I] * l.x[I] + mg_off(l, I, c, l.x.data())); });
    MGLevel& cl = g_mg.lv[k + 1];
    const G& gc = cl.g;
    const int nz = gc.D == 3 ? 2 : 1;
    inside(gc, [&](long Ic, const long* c) {
        long fb[3] = {2 * c[0] - 1, 2 * c[1] - 1, gc.D == 3 ? 2 * c[2] - 1 : 0};
        double acc = 0;
        for (int dz = 0; dz < nz; ++dz)
            for (int dy = 0; dy < 2; ++dy)
                for (int dx = 0; dx < 2; ++dx) acc += l.r[g.lin(fb) + dx + dy * g.s[1] + dz * g.s[2]];
        cl.b[Ic] = acc;
    });
    mg_vcycle(k + 1, nu1, nu2, nuc);
    inside(g, [&](long I, const long* c) {
        long cc[3] = {(c[0] + 1) / 2, (c[1] + 1) / 2, g.D == 3 ? (c[2] + 1) / 2 : 0};
        l.x[I] += cl.x[gc.lin(cc)];
    });
    for (int it = 0; it < nu2; ++it) { mg_rbgs(l, 1); mg_rbgs(l, 0); }
}
void poisson_mg_fcg(const G& g, orc_state* s) {
    double *x = s->p, *L = s->mu0;
    set_diag(g, s);
    mg_build(g, L);
    std::vector<double>& r = g_mg.r;
    std::vector<double>& rold = g_mg.rold;
    std::vector<double>& sv = g_mg.sv;
    std::vector<double>& p = g_mg.p;
    std::vector<double>& q = g_mg.q;
    MGLevel& l0 = g_mg.lv[0];
    const int nu1 = 2, nu2 = 2;
    long coarse = 1;
    for (int e = 0; e < g.D; ++e) coarse *= g_mg.lv.back().g.n[e] - 2;
    const int nuc = int(std::min<long>(4000, std::max<long>(16, 4 * coarse)));
    auto true_resid = [&]() {
        perbc(g, x);
        inside(g, [&](long I, const long*) { r[I] = s->sigma[I] - mult(g, I, L, s->pD, x); });
        return linf_inside(g, r.data());
    };
    double res = true_resid();
    int it = 0;
    double sr_old = 0;
    while (res > s->ptol && it < s->pitmx) {
        std::copy(r.begin(), r.end(), l0.b.begin());
        mg_vcycle(0, nu1, nu2, nuc);
        std::copy(l0.x.begin(), l0.x.end(), sv.begin());
        const double sr = dot_inside(g, sv.data(), r.data());
        if (it == 0) {
            inside(g, [&](long I, const long*) { p[I] = sv[I]; });
        } else {
            double num = 0;
            {
                long lo[3] = {1, 1, 1}, hi[3] = {g.n[0] - 2, g.n[1] - 2, g.n[2] - 2};
                if (g.D == 2) lo[2] = hi[2] = 0;
#pragma omp parallel for collapse(2) reduction(+ : num)
                for (long kk = lo[2]; kk <= hi[2]; ++kk)
                    for (long j = lo[1]; j <= hi[1]; ++j)
                        for (long i = lo[0]; i <= hi[0]; ++i) {
                            long I = i + g.s[1] * j + g.s[2] * kk;
                            num += sv[I] * (r[I] - rold[I]);
                        }
            }
            const double beta = num / sr_old;
            inside(g, [&](long I, const long*) { p[I] = sv[I] + beta * p[I]; });
        }
        perbc(g, p.data());
        inside(g, [&](long I, const long*) { q[I] = mult(g, I, L, s->pD, p.data()); });
        const double alpha = sr / dot_inside(g, p.data(), q.data());
        std::copy(r.begin(), r.end(), rold.begin());
        inside(g, [&](long I, const long*) {
            x[I] += alpha * p[I];
            r[I] -= alpha * q[I];
        });
        sr_old = sr;
        ++it;
        res = linf_inside(g, r.data());
        if (res <= s->ptol) res = true_resid();
    }
    perbc(g, x);
    s->piters = it;
    s->presid = res;
}
void poisson(const G& g, orc_state* s) {
    if (s->psolver == ORC_POISSON_MG) poisson_mg_fcg(g, s);
    else poisson_jacobi_pcg(g, s);
}
// myproject! / inproject!, flow.jl:328-347 (source z = σ, x = p, L = μ₀)
void project(const G& g, orc_state* s, double w, double dt_last) {
    double dt = w * dt_last;
    inside(g, [&](long I, const long*) { s->sigma[I] = divu(g, I, s->u); });
    for (long k = 0; k < g.N; ++k) s->p[k] *= dt;
    poisson(g, s);
    for (int i = 0; i < g.D; ++i)
        inside(g, [&](long I, const long*) {
            s->u[I + i * g.N] -= s->mu0[I + i * g.N] * (s->p[I] - s->p[I - g.s[i]]);
        });
    for (long k = 0; k < g.N; ++k) s->p[k] *= 1 / dt;
}

// viscSurfTenρu!, flow.jl:113-117
void visc_surften(const G& g, orc_state* s, const double* f) {
    std::fill(s->force, s->force + g.D * g.N, 0.0);
    if (s->mu != 0) visc(g, s->force, s->u, s->nhat, s->sigma, f, s->lmu, s->mu, s->lrho);
    if (s->eta != 0) surften(g, s->force, f, s->nhat, s->fF, s->eta);
}

// maxTotalFlux, flow.jl:283-289 ; WaterLily flux_out
inline double max_total_flux(const G& g, long I, const double* u) {
    double sm = 0;
    for (int i = 0; i < g.D; ++i) sm += jmax(std::fabs(u[I + i * g.N]), std::fabs(u[I + g.s[i] + i * g.N]));
    return sm;
}
inline double flux_out(const G& g, long I, const double* u) {
    double sm = 0;
    for (int i = 0; i < g.D; ++i) sm += jmax(0.0, u[I + g.s[i] + i * g.N]) + jmax(0.0, -u[I + i * g.N]);
    return sm;
}
// MPCFL, flow.jl:262-281 (σ scratch: zero then interior values, maximum over the whole array)
double mpcfl(const G& g, orc_state* s) {
    std::fill(s->sigma, s->sigma + g.N, 0.0);
    inside(g, [&](long I, const long*) { s->sigma[I] = flux_out(g, I, s->u); });
    double m1 = *std::max_element(s->sigma, s->sigma + g.N);
    double dtAdv = 1 / (m1 + 5 * s->nu);
    inside(g, [&](long I, const long*) { s->sigma[I] = max_total_flux(g, I, s->u); });
    double m2 = *std::max_element(s->sigma, s->sigma + g.N);
    double dtV = 1 / (2 * m2);
    double dtG = 1.0, dtVisc = 1.0, dtST = 1.0;
    if (s->has_g) {
        double g2 = 0;
        for (int i = 0; i < g.D; ++i) g2 += s->g[i] * s->g[i];
        dtG = 1 / (2 * std::sqrt(g2));
    }
    if (s->mu != 0) dtVisc = 3 / (14 * s->mu * jmax(1.0, s->lmu / s->lrho));
    if (s->eta != 0) dtST = std::sqrt((1 + s->lrho) / (8 * M_PI * s->eta));
    return 0.8 * jmin(jmin(jmin(dtV, dtAdv), jmin(dtG, dtVisc)), dtST);
}

// MPFMomStep!, flow.jl:60-109.  dt = δt, t1 = sum(Δt), n_dt = length(Δt) (sets dirO).
void mom_step(const G& g, orc_state* s, double dt, double t1, long n_dt, orc_fill_status* st) {
    (void)t1;
    long NV = g.D * g.N;
    int dirO[3];
    for (int i = 1; i <= g.D; ++i) dirO[i - 1] = int((n_dt + i) % g.D);   // flow.jl:163
    std::memcpy(s->u0, s->u, sizeof(double) * NV);
    std::memcpy(s->f0, s->f, sizeof(double) * g.N);
    // predictor
    u2rhou(g, s->rhou, s->u0, s->f0, s->lrho);
    bc_vel(g, s->rhou, s->uBC);
    advect_vof_rhouu(g, s, s->f0, s->u0, s->u, s->u, dt, dirO, st);
    std::fill(s->mu0, s->mu0 + NV, 1.0);
    for (long k = 0; k < g.N; ++k) s->f0[k] = (s->f0[k] + s->f[k]) / 2;
    visc_surften(g, s, s->f0);
    u2rhou(g, s->nhat, s->u0, s->f, s->lrho);
    update_u(g, s, s->u, s->rhou, s->nhat, s->force, dt, s->f0, 0.5);
    bc_vel(g, s->u, s->uBC);
    update_L(g, s, s->f0);
    project(g, s, 0.5, dt);
    bc_vel(g, s->u, s->uBC);
    // corrector
    std::memcpy(s->f0, s->f, sizeof(double) * g.N);
    u2rhou(g, s->rhou, s->u0, s->f, s->lrho);
    bc_vel(g, s->rhou, s->uBC);
    advect_vof_rhouu(g, s, s->f, s->u, s->u, s->u0, dt, dirO, st);
    std::fill(s->mu0, s->mu0 + NV, 1.0);
    visc_surften(g, s, s->f);
    u2rhou(g, s->nhat, s->u0, s->f, s->lrho);
    std::memcpy(s->u0, s->u, sizeof(double) * NV);
    update_u(g, s, s->u, s->rhou, s->nhat, s->force, dt, s->f, 1.0);
    bc_vel(g, s->u, s->uBC);
    update_L(g, s, s->f);
    project(g, s, 1.0, dt);
    bc_vel(g, s->u, s->uBC);
}

}  // namespace

/* ===================== exported C-ABI ===================== */
extern "C" {

double orc_get_intercept2(double n1, double n2, double g) { return get_intercept(n1, n2, g); }
double orc_get_intercept3(double n1, double n2, double n3, double g) { return get_intercept(n1, n2, n3, g); }
double orc_get_volume_fraction2(double n1, double n2, double b) { return get_vf(n1, n2, b); }
double orc_get_volume_fraction3(double n1, double n2, double n3, double b) { return get_vf(n1, n2, n3, b); }
float orc_get_intercept2f(float n1, float n2, float g) { return get_intercept(n1, n2, g); }
float orc_get_intercept3f(float n1, float n2, float n3, float g) { return get_intercept(n1, n2, n3, g); }
float orc_get_volume_fraction2f(float n1, float n2, float b) { return get_vf(n1, n2, b); }
float orc_get_volume_fraction3f(float n1, float n2, float n3, float b) { return get_vf(n1, n2, n3, b); }
double orc_proot(double c0, double c1, double c2, double c3) { return proot(c0, c1, c2, c3); }

int orc_normal(const orc_grid* gg, int scheme, const double* f, double* nhat, int64_t I) {
    G g(gg);
    double n[3];
    if (!normal(g, scheme, f, I, n)) return -1;
    for (int d = 0; d < g.D; ++d) nhat[I + d * g.N] = n[d];
    return 0;
}
void orc_reconstruct(const orc_grid* gg, int scheme, const double* f, double* alpha, double* nhat) {
    G g(gg);
    reconstruct(g, scheme, const_cast<double*>(f), alpha, nhat);
}
void orc_bcvof(const orc_grid* gg, double* f, double* alpha, double* nhat) { bcvof(G(gg), f, alpha, nhat); }
void orc_bcf(const orc_grid* gg, double* f) { bcf(G(gg), f); }
void orc_bcf_d(const orc_grid* gg, int d, double* f) { bcf_d(G(gg), d, f); }
void orc_bcv(const orc_grid* gg, double* v) { bcv(G(gg), v); }
void orc_bc_vel(const orc_grid* gg, double* a, const double* A) { bc_vel(G(gg), a, A); }
void orc_perbc(const orc_grid* gg, double* x) { perbc(G(gg), x); }
void orc_clean_wisp(const orc_grid* gg, double* f, double tol) { clean_wisp(G(gg), f, tol); }
void orc_f2face(const orc_grid* gg, double* ff, const double* f) { f2face(G(gg), ff, f); }
double orc_get3cellheight(const orc_grid* gg, const double* f, int64_t I, int s) { return h3(G(gg), f, I, s); }
double orc_getmu(const orc_grid* gg, int i, int j, int64_t I, const double* ff, double lmu, double mu, double lrho) {
    return getmu(G(gg), i, j, I, ff, lmu, mu, lrho);
}

// applyVOF!, VOFutil.jl:9-37 (then cleanWisp!); Δx = 0.01 finite differences supplied as samples
void orc_apply_vof(const orc_grid* gg, double* f, double* alpha, double* nhat, const double* const* sdf) {
    G g(gg);
    inside(g, [&](long I, const long*) {
        double sumN = 0, sumN2 = 0, n[3] = {0, 0, 0};
        for (int i = 0; i < g.D; ++i) {
            double dd = sdf[1 + 2 * i][I] - sdf[2 + 2 * i][I];
            n[i] = dd;
            nhat[I + i * g.N] = dd;
            sumN += dd;
            sumN2 += dd * dd;
        }
        alpha[I] = sumN / 2 - std::sqrt(sumN2) * sdf[0][I];
        f[I] = vf_D(g.D, n, alpha[I]);
    });
    clean_wisp(g, f, 10 * 2.220446049250313e-16);
}

void orc_vof_flux(const orc_grid* gg, double* fF, const double* f, const double* alpha, const double* nhat,
                  const double* u, const double* u0, double dt, int d, double* rhouf, double lrho) {
    vof_flux(G(gg), fF, f, alpha, nhat, u, u0, dt, d, rhouf, lrho);
}

// advectVOF!, advection.jl:34-78 (Lie–Trotter; dirO 0-based)
void orc_advect_vof(const orc_grid* gg, int scheme, double* f, double* fF, double* alpha, double* nhat,
                    const double* u, const double* u0, double dt, int8_t* cbar, double* rhouf, double lrho,
                    const int* dirO, orc_fill_status* st) {
    G g(gg);
    const double tol = 10 * 2.220446049250313e-16;
    std::fill(rhouf, rhouf + g.D * g.N, 0.0);
    allcells(g, [&](long I, const long*) { cbar[I] = f[I] < 0.5 ? 0 : 1; });
    for (int k = 0; k < g.D; ++k)
        advect_vof_1d(g, scheme, f, fF, alpha, nhat, u, u0, dt, cbar, rhouf, lrho, dirO[k], tol, tol, st);
}

void orc_surften(const orc_grid* gg, double* forcing, const double* f, double* nhat, double* fbuffer, double eta) {
    surften(G(gg), forcing, f, nhat, fbuffer, eta);
}
double orc_popinet_height(const orc_grid* gg, const double* f, int64_t I, int i_signed) {
    return popinet_height(G(gg), f, I, i_signed);
}
double orc_curvature(const orc_grid* gg, const double* f, int64_t I, int i_signed) {
    return curvature(G(gg), f, I, i_signed);
}

void orc_mom_step(const orc_grid* gg, orc_state* s, double dt, double t_now, int64_t n_dt, orc_fill_status* st) {
    mom_step(G(gg), s, dt, t_now, n_dt, st);
}
double orc_mpcfl(const orc_grid* gg, orc_state* s, double) { return mpcfl(G(gg), s); }
void orc_poisson(const orc_grid* gg, orc_state* s) { poisson(G(gg), s); }


/* small helpers exported for the known-answer tests of src/util.jl and src/VOFutil.jl */
int orc_argabsmax(int D, const double* n) { return argabsmax(D, n); }
int orc_get_xdir(int i) { return get_xdir(i); }
void orc_get_xydir(int i, int* ix, int* iy) { get_xydir(i, *ix, *iy); }
double orc_getrho_cell(double f, double lrho) { return lin_prop(f, lrho); }
double orc_getrho_face(const orc_grid* gg, int d, int64_t I, const double* f, double lrho) {
    return rho_face(G(gg), d, I, f, lrho);
}
// per-face getVOFFlux!(fᶠ,f,α,n̂,δl,d,IFace,ρuf,λρ), advection.jl:113-137
void orc_vof_flux_face(const orc_grid* gg, double* fF, const double* f, const double* al, const double* nh, double dl,
                       int d, int64_t IF, double* rhouf, double lrho) {
    G g(gg);
    if (dl == 0) return;
    long IC = dl > 0 ? IF - g.s[d] : IF;
    double sa = 0;
    for (int ii = 0; ii < g.D; ++ii) sa += std::fabs(nh[IC + ii * g.N]);
    if (sa == 0 || fullorempty(f[IC])) {
        fF[IF] = f[IC] * dl;
    } else {
        double a = dl > 0 ? al[IC] - nh[IC + d * g.N] * (1 - dl) : al[IC];
        double nc[3] = {0, 0, 0};
        for (int ii = 0; ii < g.D; ++ii) nc[ii] = nh[IC + ii * g.N] * (ii == d ? std::fabs(dl) : 1.0);
        fF[IF] = vf_D(g.D, nc, a) * dl;
    }
    rhouf[IF + d * g.N] += dl * lrho + (1 - lrho) * fF[IF];
}

}  // extern "C"
