// ORACLE — test infrastructure, not product code.
//
// CPU restatement of the per-cell diagnostics of src/metrics.jl and their domain sums, in the
// reference's layout (column-major, one ghost layer, vectors component-last, 0-based indices).
// Pinned by the known answers of test/maintests.jl:321-347 (tests/test_metrics_cpu.py).
#include <cstdint>

#include "oracle.h"

namespace {

int64_t stride(const orc_grid* g, int d) {
    int64_t s = 1;
    for (int e = 0; e < d; ++e) s *= g->n[e];
    return s;
}
int64_t total(const orc_grid* g) { return g->n[0] * g->n[1] * (g->D == 3 ? g->n[2] : 1); }

// getρ(I,f,λρ) = linInterpProp(f[I],λρ) (src/VOFutil.jl:166,174)
double rho_cell(const double* f, int64_t I, double lrho) { return f[I] + (1.0 - f[I]) * lrho; }

}  // namespace

extern "C" {

// ρkeI(I,u,f,λρ,U), src/metrics.jl:13-15
double orc_rhoke(const orc_grid* g, int64_t I, const double* u, const double* f, double lrho, const double* U) {
    const int64_t N = total(g);
    double s = 0.0;
    for (int i = 0; i < g->D; ++i) {
        const double a = u[I + i * N] - U[i], b = u[I + stride(g, i) + i * N] - U[i];
        s += a * a + b * b;
    }
    return 0.25 * s * rho_cell(f, I, lrho);
}

// ρuI(i,I,u,f,λρ,U), src/metrics.jl:56-58
double orc_rhou(const orc_grid* g, int i, int64_t I, const double* u, const double* f, double lrho,
                const double* U) {
    const int64_t N = total(g);
    return 0.5 * (u[I + i * N] + u[I + stride(g, i) + i * N] - 2.0 * U[i]) * rho_cell(f, I, lrho);
}

// ρgh(I,g,f,λρ,StatWL), src/metrics.jl:23, with loc(0,I) = I - 1.5 (1-based) = c - 0.5 (0-based)
double orc_rhogh(const orc_grid* g, int64_t I, const double* gv, const double* f, double lrho,
                 const double* wl) {
    double s = 0.0;
    int64_t r = I;
    for (int i = 0; i < g->D; ++i) {
        const int64_t c = r % g->n[i];
        r /= g->n[i];
        s += gv[i] * ((double(c) - 0.5) - wl[i]);
    }
    return -rho_cell(f, I, lrho) * s;
}

// EnsI(I,ω), src/metrics.jl:32-39 (3D: ω component i read at I, I+δix, I+δiy, I+δix+δiy with
// ix, iy = shiftDir(i,3,1), shiftDir(i,3,2); 2D: scalar ω at the four corners)
double orc_ens(const orc_grid* g, int64_t I, const double* w) {
    double s = 0.0;
    if (g->D == 3) {
        const int64_t N = total(g);
        for (int i = 0; i < 3; ++i) {
            const int64_t sx = stride(g, (i + 1) % 3), sy = stride(g, (i + 2) % 3);
            const double* wi = w + i * N;
            s += wi[I] * wi[I] + wi[I + sx] * wi[I + sx] + wi[I + sy] * wi[I + sy] +
                 wi[I + sx + sy] * wi[I + sx + sy];
        }
    } else {
        const int64_t sx = stride(g, 0), sy = stride(g, 1);
        s = w[I] * w[I] + w[I + sx] * w[I + sx] + w[I + sy] * w[I + sy] + w[I + sx + sy] * w[I + sx + sy];
    }
    return 0.5 * 0.25 * s;
}

// sums over interior cells: out = {Σρke, Σρgh, ΣEns (0 without ω), Σρu_0, .., Σρu_{D-1}}
void orc_metrics(const orc_grid* g, const double* u, const double* f, const double* w, double lrho,
                 const double* U, const double* gv, const double* wl, double* out) {
    for (int q = 0; q < 3 + g->D; ++q) out[q] = 0.0;
    const int64_t nz = g->D == 3 ? g->n[2] : 3;
    for (int64_t z = 1; z < nz - 1; ++z)
        for (int64_t y = 1; y < g->n[1] - 1; ++y)
            for (int64_t x = 1; x < g->n[0] - 1; ++x) {
                const int64_t I = x + g->n[0] * (y + (g->D == 3 ? g->n[1] * z : 0));
                out[0] += orc_rhoke(g, I, u, f, lrho, U);
                out[1] += orc_rhogh(g, I, gv, f, lrho, wl);
                if (w) out[2] += orc_ens(g, I, w);
                for (int i = 0; i < g->D; ++i) out[3 + i] += orc_rhou(g, i, I, u, f, lrho, U);
            }
}

}  // extern "C"
