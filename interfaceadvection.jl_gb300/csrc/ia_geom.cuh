// Interface geometry on the device, FP64: the PLIC plane-constant solve
// (Scardovelli & Zaleski 2000, as used by src/PLIC.jl) and the interface-normal
// schemes of src/normalEstimation.jl.
//
// Conventions shared with the reference: the dark fluid has f = 1, the normal
// n̂ points into the light fluid and is not unit-normalised; a cell holds the
// dark region {x : n̂·(x - corner) < α}.
#pragma once
#include "ia_core.cuh"

namespace ia {

// ------------------------------------------------------------------ PLIC

// Sorted, |n|-normalised magnitudes m1 <= m2 (<= m3) of a normal.
__device__ __forceinline__ void plic_sort(double& a, double& b) {
    if (!(a < b)) { double t = a; a = b; b = t; }
}
__device__ __forceinline__ void plic_sort(double& a, double& b, double& c) {
    if (a > c) { double t = a; a = c; c = t; }
    if (a > b) { double t = a; a = b; b = t; }
    if (b > c) { double t = b; b = c; c = t; }
}

// Volume below the plane m·x = a inside the unit square/cube, for m >= 0,
// Σm = 1 and a <= 1/2 (src/PLIC.jl:92-107).
__device__ __forceinline__ double plic_volume(double m1, double m2, double a) {
    return a < m1 ? a * a / (2.0 * m1 * m2) : (a - 0.5 * m1) / m2;
}
__device__ inline double plic_volume(double m1, double m2, double m3, double a) {
    const double m12 = m1 + m2;
    const double p6 = 6.0 * m1 * m2 * m3;
    if (a < m1) return a * a * a / p6;
    if (a < m2) {
        // the (m2 == 0) guard keeps the m1 = m2 = 0 column finite (PLIC.jl:99)
        const double r = (m2 == 0.0) ? 1.0 : m1 / m2;
        return a * (a - m1) / (2.0 * m2 * m3) + r * m1 / (6.0 * m3);
    }
    const double c12 = m1 * m1 * (m1 - 3.0 * a) + m2 * m2 * (m2 - 3.0 * a);
    if (a < fmin(m3, m12)) return (a * a * (3.0 * m12 - a) + c12) / p6;
    if (m3 < m12) return (a * a * (3.0 - 2.0 * a) + c12 + m3 * m3 * (m3 - 3.0 * a)) / p6;
    return (2.0 * a - m12) / (2.0 * m3);
}

// Real root of c3 x^3 + c2 x^2 + c1 x + c0 selected by the trigonometric
// form used in src/PLIC.jl:165-176.
__device__ inline double plic_cubic_root(double c0, double c1, double c2, double c3) {
    const double a0 = c0 / c3, a1 = c1 / c3, a2 = c2 / c3;
    const double p0 = a1 / 3.0 - a2 * a2 / 9.0;
    const double q0 = (a1 * a2 - 3.0 * a0) / 6.0 - a2 * a2 * a2 / 27.0;
    double a = q0 / sqrt(-p0 * p0 * p0);
    a = (a * a <= 1.0) ? a : 0.0;
    const double t = acos(a) / 3.0;
    double st, ct;
    sincos(t, &st, &ct);
    return sqrt(-p0) * (sqrt(3.0) * st - ct) - a2 / 3.0;
}

// Plane constant for volume v <= 1/2 (src/PLIC.jl:117-149).
__device__ __forceinline__ double plic_intercept(double m1, double m2, double v) {
    return v < m1 / (2.0 * m2) ? sqrt(2.0 * m1 * m2 * v) : m2 * v + 0.5 * m1;
}
__device__ inline double plic_intercept(double m1, double m2, double m3, double v) {
    const double m12 = m1 + m2;
    const double p = 6.0 * m1 * m2 * m3;
    const double v1 = ((m2 == 0.0) ? 1.0 : m1 / m2) * m1 / (6.0 * m3);
    const double v2 = v1 + (m2 - m1) / (2.0 * m3);
    const double v3 = (m3 < m12)
                          ? (m3 * m3 * (3.0 * m12 - m3) + m1 * m1 * (m1 - 3.0 * m3) + m2 * m2 * (m2 - 3.0 * m3)) / p
                          : m12 / (2.0 * m3);
    if (v < v1) return cbrt(p * v);
    if (v < v2) return 0.5 * (m1 + sqrt(m1 * m1 + 8.0 * m2 * m3 * (v - v1)));
    if (v < v3)
        return plic_cubic_root(m1 * m1 * m1 + m2 * m2 * m2 - p * v, -3.0 * (m1 * m1 + m2 * m2), 3.0 * m12, -1.0);
    if (m3 < m12)
        return plic_cubic_root(m1 * m1 * m1 + m2 * m2 * m2 + m3 * m3 * m3 - p * v,
                               -3.0 * (m1 * m1 + m2 * m2 + m3 * m3), 3.0, -2.0);
    return m3 * v + 0.5 * m12;
}

// getIntercept (src/PLIC.jl:20-39): α of the cell with normal n and fraction g.
template <int D>
__device__ double get_intercept(const double n[3], double g) {
    double t = fabs(n[0]) + fabs(n[1]);
    if (D == 3) t += fabs(n[2]);
    double a = 0.5;
    const double v = g < 0.5 ? g : 1.0 - g;
    if (g != 0.5) {
        double m1 = fabs(n[0]) / t, m2 = fabs(n[1]) / t;
        if (D == 2) {
            plic_sort(m1, m2);
            a = plic_intercept(m1, m2, v);
        } else {
            double m3 = fabs(n[2]) / t;
            plic_sort(m1, m2, m3);
            a = plic_intercept(m1, m2, m3, v);
        }
    }
    double shift = fmin(n[0], 0.0) + fmin(n[1], 0.0);
    if (D == 3) shift += fmin(n[2], 0.0);
    return (g < 0.5 ? a : 1.0 - a) * t + shift;
}

// getVolumeFraction (src/PLIC.jl:59-82): dark volume of a cell cut by n·x = b.
template <int D>
__device__ double get_volume_fraction(const double n[3], double b) {
    double t = fabs(n[0]) + fabs(n[1]);
    double shift = fmin(n[0], 0.0) + fmin(n[1], 0.0);
    if (D == 3) {
        t += fabs(n[2]);
        shift += fmin(n[2], 0.0);
    }
    // (b - min(n1,0) - min(n2,0) - ...) evaluated left to right
    double a = b - fmin(n[0], 0.0) - fmin(n[1], 0.0);
    if (D == 3) a -= fmin(n[2], 0.0);
    a /= t;
    (void)shift;
    if (a <= 0.0 || a == 0.5 || a >= 1.0) return fmin(fmax(a, 0.0), 1.0);
    const double w = a < 0.5 ? a : 1.0 - a;
    double m1 = fabs(n[0]) / t, m2 = fabs(n[1]) / t, v;
    if (D == 2) {
        plic_sort(m1, m2);
        v = plic_volume(m1, m2, w);
    } else {
        double m3 = fabs(n[2]) / t;
        plic_sort(m1, m2, m3);
        v = plic_volume(m1, m2, m3, w);
    }
    return a < 0.5 ? v : 1.0 - v;
}

// ------------------------------------------------------------------ normals
//
// A read-only view of the fraction field around one cell.  All neighbour
// reads stay inside the 3x3(x3) box of the cell, whose ghosts are valid.
struct Stencil {
    const double* __restrict__ f;
    long long c;        // centre cell
    long long s[3];     // strides
    __device__ __forceinline__ double at(long long off) const { return __ldg(f + c + off); }
    // Three-cell column sum through c + off along axis a (get3CellHeight, src/VOFutil.jl:158)
    __device__ __forceinline__ double col3(long long off, int a) const {
        return at(off) + at(off - s[a]) + at(off + s[a]);
    }
};

__device__ __forceinline__ double jl_sign(double x) { return x > 0.0 ? 1.0 : (x < 0.0 ? -1.0 : x); }
__device__ __forceinline__ double sign_or_one(double x) { const double s = jl_sign(x); return s == 0.0 ? 1.0 : s; }

// Index of the first component with the strictly largest |n| (myArgAbsMax, src/util.jl:19-31).
template <int D>
__device__ __forceinline__ int arg_abs_max(const double n[3]) {
    int im = 0;
    double mx = 0.0;
#pragma unroll
    for (int i = 0; i < D; ++i) {
        const double c = n[i] * n[i];
        if (c > mx) { mx = c; im = i; }
    }
    return im;
}

// central difference of f (PCD)
template <int D>
__device__ __forceinline__ void normal_pcd(const Stencil& S, double n[3]) {
#pragma unroll
    for (int d = 0; d < D; ++d) n[d] = S.at(-S.s[d]) - S.at(S.s[d]);
}

// PCD guess, then centred column-height differences across the dominant axis.
// steep = true adds the Weymouth–Yue one-sided switch (WY); false is Column.
template <int D, bool steep>
__device__ void normal_columns(const Stencil& S, double n[3]) {
    normal_pcd<D>(S, n);
    const int dom = arg_abs_max<D>(n);
#pragma unroll
    for (int d = 0; d < D; ++d) {
        if (d == dom) { n[d] = sign_or_one(n[d]); continue; }
        const double hl = S.col3(-S.s[d], dom), hr = S.col3(S.s[d], dom);
        double v = 0.5 * (hl - hr);
        if (steep && fabs(v) > 0.5) {
            const double hc = S.col3(0, dom);
            v = (v * (hc - 1.5) >= 0.0) ? hc - hr : hl - hc;
        }
        n[d] = v;
    }
}

// Huang–Weymouth: Column estimate normalised by its dominant component, with
// row-width corrections where the three column heights leave the range a
// straight interface of that slope can produce (src/normalEstimation.jl:105-154).
template <int D>
__device__ void normal_wh(const Stencil& S, double n[3]) {
    normal_columns<D, false>(S, n);
    const int ad = arg_abs_max<D>(n);
    const long long dstep = signbit(n[ad]) ? -S.s[ad] : S.s[ad];
    double an = fabs(n[ad]);
    an = (an == 0.0) ? 1.0 : an;
#pragma unroll
    for (int d = 0; d < D; ++d) n[d] /= an;
#pragma unroll
    for (int d = 0; d < D; ++d) {
        if (d == ad) continue;
        const double slope = fabs(n[d]);
        const bool neg = signbit(n[d]);
        const long long step = neg ? -S.s[d] : S.s[d];
        const double hl = S.col3(-step, ad), hc = S.col3(0, ad), hr = S.col3(step, ad);
        const double sh = hl + hc + hr;
        const double tri = 4.5 * slope;
        if (tri <= sh && sh <= 9.0 - tri) continue;
        const double lim = fmin(1.0 / (2.0 * slope), tri);
        const double sgn = neg ? -1.0 : 1.0;
        if (sh < tri) {
            const double wb = S.col3(-dstep, d);
            if (wb > lim) n[d] = copysign((hl - 0.5) / (wb - 0.5), sgn);
        }
        if (sh > 9.0 - tri) {
            const double wt = S.col3(dstep, d);
            if (wt < 3.0 - lim) n[d] = copysign((2.5 - hr) / (2.5 - wt), sgn);
        }
    }
}

template <int D>
__device__ void normal_slic(const Stencil& S, double n[3]) {
    normal_pcd<D>(S, n);
    const int dd = arg_abs_max<D>(n);
#pragma unroll
    for (int i = 0; i < D; ++i) n[i] = (i == dd) ? jl_sign(n[i]) : 0.0;
}

// Youngs' weighted (1-2-1) face sum over the plane through c+off normal to d,
// accumulated in the reference's CartesianIndices order (src/normalEstimation.jl:248-257).
template <int D>
__device__ double young_sum(const Stencil& S, long long off, int d) {
    double a = 0.0;
    if (D == 2) {
        const long long e = S.s[1 - d];
        for (int ii = -1; ii <= 0; ++ii)
            for (int jj = ii; jj <= ii + 1; ++jj) a += S.at(off + jj * e);
    } else {
        const long long e0 = S.s[d == 0 ? 1 : 0], e1 = S.s[d == 2 ? 1 : 2];
        for (int i1 = -1; i1 <= 0; ++i1)
            for (int i0 = -1; i0 <= 0; ++i0)
                for (int j1 = i1; j1 <= i1 + 1; ++j1)
                    for (int j0 = i0; j0 <= i0 + 1; ++j0) a += S.at(off + j0 * e0 + j1 * e1);
    }
    return a;
}
template <int D>
__device__ void normal_young(const Stencil& S, double n[3]) {
    double a = 0.0;
    for (int d = 0; d < D; ++d) {
        n[d] = (young_sum<D>(S, -S.s[d], d) - young_sum<D>(S, S.s[d], d)) * 0.5;
        a += fabs(n[d]);
    }
    for (int d = 0; d < D; ++d) n[d] = (a == 0.0) ? 1.0 / D : n[d] / a;
}
// centred-column estimate along dc, signed by ref (src/normalEstimation.jl:210-224)
template <int D>
__device__ void normal_cc(const Stencil& S, int dc, const double ref[3], double out[3]) {
    double s = 0.0;
    for (int d = 0; d < D; ++d) {
        out[d] = (d == dc) ? sign_or_one(ref[d]) : -(S.col3(S.s[d], dc) - S.col3(-S.s[d], dc)) / 2.0;
        s += fabs(out[d]);
    }
    for (int d = 0; d < D; ++d) out[d] /= s;
}
// mixed Youngs–centred (src/normalEstimation.jl:185-202)
template <int D>
__device__ void normal_myc(const Stencil& S, double n[3]) {
    normal_young<D>(S, n);
    double mx = 0.0;
    for (int i = 0; i < D; ++i) mx = fabs(n[i]) > mx ? fabs(n[i]) : mx;
    double prev = 0.0, tmp[3];
    int cz = 0;
    for (int iz = 0; iz < D; ++iz) {
        normal_cc<D>(S, iz, n, tmp);
        if (fabs(tmp[iz]) > prev) cz = iz;
        prev = fabs(tmp[iz]);
    }
    normal_cc<D>(S, cz, n, tmp);
    if (fabs(tmp[cz]) < mx)
        for (int i = 0; i < D; ++i) n[i] = tmp[i];
}
// nearest-neighbour cross sums (src/normalEstimation.jl:266-277)
template <int D>
__device__ double cross_sum(const Stencil& S, long long off, int d) {
    double a = S.at(off);
    for (int e = 0; e < D; ++e) a += (e != d) ? (S.at(off - S.s[e]) + S.at(off + S.s[e])) : 0.0;
    return a;
}
template <int D>
__device__ void normal_cd(const Stencil& S, double n[3]) {
    for (int d = 0; d < D; ++d) n[d] = (cross_sum<D>(S, -S.s[d], d) - cross_sum<D>(S, S.s[d], d)) * 0.5;
}

template <int D>
__device__ void interface_normal(int scheme, const Stencil& S, double n[3]) {
    n[0] = n[1] = n[2] = 0.0;
    switch (scheme) {
        case IA_NORMAL_WY: normal_columns<D, true>(S, n); break;
        case IA_NORMAL_MYC: normal_myc<D>(S, n); break;
        case IA_NORMAL_Y: normal_young<D>(S, n); break;
        case IA_NORMAL_COLUMN: normal_columns<D, false>(S, n); break;
        case IA_NORMAL_PCD: normal_pcd<D>(S, n); break;
        case IA_NORMAL_SLIC: normal_slic<D>(S, n); break;
        case IA_NORMAL_CD: normal_cd<D>(S, n); break;
        case IA_NORMAL_XYLIC:
            for (int i = 0; i < D; ++i) n[i] = (i == 1) ? 1.0 : 0.0;
            break;
        default: normal_wh<D>(S, n); break;
    }
}

}  // namespace ia
