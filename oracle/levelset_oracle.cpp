// ORACLE — test infrastructure, not product code.
//
// CPU restatement of src/redistaning.jl in the reference's layout (column-major, one ghost
// layer, 0-based): LevelSet's ϕ = 2f - 1 (:13-25), computeL! with its Neumann and periodic
// boundary building blocks (:64-110), ∇ϕᵢ² (:118-143), _redistaningStage! (:27-30) and
// redistaning! (:42-54).  Pinned by test/maintests.jl:264-319 (tests/test_levelset_cpu.py).
#include <cmath>
#include <cstdint>
#include <vector>

#include "oracle.h"

namespace {

int64_t stride(const orc_grid* g, int d) {
    int64_t s = 1;
    for (int e = 0; e < d; ++e) s *= g->n[e];
    return s;
}
int64_t total(const orc_grid* g) { return g->n[0] * g->n[1] * (g->D == 3 ? g->n[2] : 1); }

double minmod(double a, double b) { return std::fabs(a) <= std::fabs(b) ? a : b; }

double grad2(double a, double b, double c, double d, double e, double s) {
    const double dp = d - c, dm = c - b;
    const double d2p = e + c - 2 * d, d2o = d + b - 2 * c, d2m = c + a - 2 * b;
    const double dR = dp - minmod(d2p, d2o) / 2, dL = dm + minmod(d2o, d2m) / 2;
    const double wR = dR * s, wL = dL * s;
    if (wR < 0 && (wR + wL) < 0) return dR * dR;
    if (wL > 0 && (wR + wL) > 0) return dL * dL;
    return 0.0;
}

double sign(double v) { return v > 0 ? 1.0 : (v < 0 ? -1.0 : v); }

void coords(const orc_grid* g, int64_t I, int c[3]) {
    c[0] = int(I % g->n[0]);
    c[1] = int((I / g->n[0]) % g->n[1]);
    c[2] = g->D == 3 ? int(I / (g->n[0] * g->n[1])) : 0;
}

bool inside(const orc_grid* g, const int c[3]) {
    for (int e = 0; e < g->D; ++e)
        if (c[e] < 1 || c[e] > g->n[e] - 2) return false;
    return true;
}

}  // namespace

extern "C" {

void orc_levelset_init(const orc_grid* g, const double* f, double* phi, double* ini) {
    for (int64_t q = 0; q < total(g); ++q) {
        phi[q] = 2 * f[q] - 1;
        if (ini) ini[q] = phi[q];
    }
}

// computeL!(L, ϕ, ϕini; perdir): per direction the lower boundary, inner and upper boundary
// loops add ∇ϕᵢ², then L = ϕini (1 - √L) over inside
void orc_levelset_rhs(const orc_grid* g, double* L, const double* phi, const double* ini) {
    const int64_t N = total(g);
    for (int64_t q = 0; q < N; ++q) L[q] = 0.0;
    for (int i = 0; i < g->D; ++i) {
        const int64_t si = stride(g, i);
        const bool per = (g->per >> i) & 1;
        const int n = int(g->n[i]);
        for (int64_t I = 0; I < N; ++I) {
            int c[3];
            coords(g, I, c);
            if (!inside(g, c)) continue;
            const int ci = c[i];
            double a = 0, e = 0;
            const double b = phi[I - si], cc = phi[I], d = phi[I + si];
            if (ci == 1) {                      // lowerL!
                a = per ? phi[I + int64_t(n - 3 - ci) * si] : b;
                e = phi[I + 2 * si];
            } else if (ci == n - 2) {           // upperL!
                a = phi[I - 2 * si];
                e = per ? phi[I + int64_t(2 - ci) * si] : d;
            } else {
                a = phi[I - 2 * si];
                e = phi[I + 2 * si];
            }
            L[I] += grad2(a, b, cc, d, e, sign(ini[I]));
        }
    }
    for (int64_t I = 0; I < N; ++I) {
        int c[3];
        coords(g, I, c);
        if (inside(g, c)) L[I] = ini[I] * (1 - std::sqrt(L[I]));
    }
}

// _redistaningStage!(ϕ, ϕ⁰, ϕini, L, dτ, α)
void orc_levelset_stage(const orc_grid* g, double* phi, const double* phi0, const double* ini, double* L,
                        double dtau, double alpha) {
    orc_levelset_rhs(g, L, phi, ini);
    for (int64_t I = 0; I < total(g); ++I) {
        int c[3];
        coords(g, I, c);
        if (inside(g, c)) phi[I] = alpha * phi0[I] + (1 - alpha) * (phi[I] + dtau * L[I]);
    }
}

// redistaning!(ls; d, dτ): round(d/dτ) SSP-RK3 steps, BCf!(ϕ) after every stage
void orc_redistance(const orc_grid* g, double* phi, double* phi0, const double* ini, double* L, double d,
                    double dtau) {
    const int64_t itmx = std::llrint(d / dtau);
    const double al[3] = {0.0, 3.0 / 4.0, 1.0 / 3.0};
    for (int64_t it = 0; it < itmx; ++it) {
        for (int64_t q = 0; q < total(g); ++q) phi0[q] = phi[q];
        for (int k = 0; k < 3; ++k) {
            orc_levelset_stage(g, phi, phi0, ini, L, dtau, al[k]);
            orc_bcf(g, phi);
        }
    }
}

}  // extern "C"
