// ORACLE — test infrastructure, not product code.
//
// FP64 CPU restatement of the learned Poisson preconditioner's network
// (interfaceadvection.jl_gb300/csrc/nn.cuh): forward pass, MSE loss and the
// full backward pass by reverse-mode differentiation, written as plain loops.
// The reference has no learned component, so this oracle is pinned by central
// finite differences of its own loss (tests/test_nn_cpu.py) and by an
// independent restatement with torch CPU conv3d / avg_pool3d / nearest
// upsampling; the GPU training and tensor-core kernels are then checked
// against it.
//
// Tensors: channels-last with a one-cell zero halo, [B][nz+2][ny+2][nx+2][C];
// parameters per layer W[27][Cout][Cin] (tap = (dz+1)*9 + (dy+1)*3 + (dx+1))
// then b[Cout].
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

constexpr int NL = 6;
constexpr int CIN[NL] = {4, 16, 32, 32, 32, 16};
constexpr int COUT[NL] = {16, 32, 32, 32, 16, 1};

long long woff(int l) {
    long long o = 0;
    for (int k = 0; k < l; ++k) o += 27LL * COUT[k] * CIN[k] + COUT[k];
    return o;
}
long long boff(int l) { return woff(l) + 27LL * COUT[l] * CIN[l]; }

struct Dm {
    int B, nx, ny, nz;
    long long padded() const { return (long long)B * (nx + 2) * (ny + 2) * (nz + 2); }
    long long pos(int b, int x, int y, int z) const {
        return (((long long)b * (nz + 2) + z + 1) * (ny + 2) + y + 1) * (nx + 2) + x + 1;
    }
    long long tap(int t) const {
        const int dx = t % 3 - 1, dy = (t / 3) % 3 - 1, dz = t / 9 - 1;
        return ((long long)dz * (ny + 2) + dy) * (nx + 2) + dx;
    }
    Dm half() const { return Dm{B, nx / 2, ny / 2, nz / 2}; }
};

using V = std::vector<double>;

#define FOR_INTERIOR(d)                         \
    for (int b = 0; b < (d).B; ++b)             \
        for (int z = 0; z < (d).nz; ++z)        \
            for (int y = 0; y < (d).ny; ++y)    \
                for (int x = 0; x < (d).nx; ++x)

V zeros(const Dm& d, int C) { return V((size_t)(d.padded() * C), 0.0); }

// Z = conv(X) + b
void conv(const Dm& d, int CI, int CO, const V& X, const double* W, const double* bias, V& Z) {
    FOR_INTERIOR(d) {
        const long long p = d.pos(b, x, y, z);
        for (int o = 0; o < CO; ++o) {
            double acc = bias[o];
            for (int t = 0; t < 27; ++t) {
                const long long q = p + d.tap(t);
                for (int c = 0; c < CI; ++c) acc += W[((long long)t * CO + o) * CI + c] * X[q * CI + c];
            }
            Z[p * CO + o] = acc;
        }
    }
}

// dX = Σ_t W[t]^T dY[p - off(t)],  dW += X ⊗ dY,  db += dY
void conv_bwd(const Dm& d, int CI, int CO, const V& X, const V& dY, const double* W, double* dW, double* db,
              V* dX) {
    FOR_INTERIOR(d) {
        const long long p = d.pos(b, x, y, z);
        for (int o = 0; o < CO; ++o) {
            const double g = dY[p * CO + o];
            db[o] += g;
            for (int t = 0; t < 27; ++t) {
                const long long q = p + d.tap(t);
                for (int c = 0; c < CI; ++c) {
                    dW[((long long)t * CO + o) * CI + c] += g * X[q * CI + c];
                    if (dX) (*dX)[q * CI + c] += W[((long long)t * CO + o) * CI + c] * g;
                }
            }
        }
    }
    // gradients scattered into halo cells are not part of the input: clear them
    if (dX) {
        V keep = zeros(d, CI);
        FOR_INTERIOR(d) {
            const long long p = d.pos(b, x, y, z);
            for (int c = 0; c < CI; ++c) keep[p * CI + c] = (*dX)[p * CI + c];
        }
        *dX = keep;
    }
}

void relu(const Dm& d, int C, const V& Z, V& A) {
    FOR_INTERIOR(d) {
        const long long p = d.pos(b, x, y, z);
        for (int c = 0; c < C; ++c) A[p * C + c] = Z[p * C + c] > 0.0 ? Z[p * C + c] : 0.0;
    }
}
void relu_bwd(const Dm& d, int C, const V& Z, const V& dA, V& dZ) {
    FOR_INTERIOR(d) {
        const long long p = d.pos(b, x, y, z);
        for (int c = 0; c < C; ++c) dZ[p * C + c] = Z[p * C + c] > 0.0 ? dA[p * C + c] : 0.0;
    }
}
// coarse (dims dc) = mean of the 2x2x2 children
void pool(const Dm& dc, int C, const V& in, V& out) {
    const Dm df{dc.B, 2 * dc.nx, 2 * dc.ny, 2 * dc.nz};
    FOR_INTERIOR(dc) {
        for (int c = 0; c < C; ++c) {
            double s = 0.0;
            for (int k = 0; k < 8; ++k)
                s += in[df.pos(b, 2 * x + (k & 1), 2 * y + ((k >> 1) & 1), 2 * z + (k >> 2)) * C + c];
            out[dc.pos(b, x, y, z) * C + c] = s / 8.0;
        }
    }
}
// fine (dims df) += coarse / 8
void pool_bwd_add(const Dm& df, int C, const V& dout, V& din) {
    const Dm dc = df.half();
    FOR_INTERIOR(df) {
        for (int c = 0; c < C; ++c) din[df.pos(b, x, y, z) * C + c] += dout[dc.pos(b, x / 2, y / 2, z / 2) * C + c] / 8.0;
    }
}
// fine = parent (+ skip)
void up(const Dm& df, int C, const V& in, const V* skip, V& out) {
    const Dm dc = df.half();
    FOR_INTERIOR(df) {
        const long long p = df.pos(b, x, y, z), P = dc.pos(b, x / 2, y / 2, z / 2);
        for (int c = 0; c < C; ++c) out[p * C + c] = in[P * C + c] + (skip ? (*skip)[p * C + c] : 0.0);
    }
}
// coarse = Σ children
void up_bwd(const Dm& dc, int C, const V& dout, V& din) {
    const Dm df{dc.B, 2 * dc.nx, 2 * dc.ny, 2 * dc.nz};
    FOR_INTERIOR(dc) {
        for (int c = 0; c < C; ++c) {
            double s = 0.0;
            for (int k = 0; k < 8; ++k)
                s += dout[df.pos(b, 2 * x + (k & 1), 2 * y + ((k >> 1) & 1), 2 * z + (k >> 2)) * C + c];
            din[dc.pos(b, x, y, z) * C + c] = s;
        }
    }
}

struct Acts {
    Dm f, hf, qt;
    V x0, z1, a1, p1, z2, a2, p2, z3, a3, u2, z4, a4, u1, z5, a5, out;
};

void forward(const double* w, Acts& A) {
    const Dm &f = A.f, &hf = A.hf, &qt = A.qt;
    A.z1 = zeros(f, 16); A.a1 = zeros(f, 16); A.p1 = zeros(hf, 16);
    A.z2 = zeros(hf, 32); A.a2 = zeros(hf, 32); A.p2 = zeros(qt, 32);
    A.z3 = zeros(qt, 32); A.a3 = zeros(qt, 32); A.u2 = zeros(hf, 32);
    A.z4 = zeros(hf, 32); A.a4 = zeros(hf, 32); A.u1 = zeros(f, 32);
    A.z5 = zeros(f, 16); A.a5 = zeros(f, 16); A.out = zeros(f, 1);
    conv(f, 4, 16, A.x0, w + woff(0), w + boff(0), A.z1);
    relu(f, 16, A.z1, A.a1);
    pool(hf, 16, A.a1, A.p1);
    conv(hf, 16, 32, A.p1, w + woff(1), w + boff(1), A.z2);
    relu(hf, 32, A.z2, A.a2);
    pool(qt, 32, A.a2, A.p2);
    conv(qt, 32, 32, A.p2, w + woff(2), w + boff(2), A.z3);
    relu(qt, 32, A.z3, A.a3);
    up(hf, 32, A.a3, &A.a2, A.u2);
    conv(hf, 32, 32, A.u2, w + woff(3), w + boff(3), A.z4);
    relu(hf, 32, A.z4, A.a4);
    up(f, 32, A.a4, nullptr, A.u1);
    conv(f, 32, 16, A.u1, w + woff(4), w + boff(4), A.z5);
    relu(f, 16, A.z5, A.a5);
    FOR_INTERIOR(f) {
        const long long p = f.pos(b, x, y, z);
        for (int c = 0; c < 16; ++c) A.a5[p * 16 + c] += A.a1[p * 16 + c];
    }
    conv(f, 16, 1, A.a5, w + woff(5), w + boff(5), A.out);
}

Acts make(const double* x0, int B, int nx, int ny, int nz) {
    Acts A;
    A.f = Dm{B, nx, ny, nz};
    A.hf = A.f.half();
    A.qt = A.hf.half();
    A.x0.assign(x0, x0 + A.f.padded() * 4);
    return A;
}

}  // namespace

extern "C" {

int64_t orc_nn_param_count() { return woff(NL); }

void orc_nn_forward(const double* w, const double* x0, int B, int nx, int ny, int nz, double* out) {
    Acts A = make(x0, B, nx, ny, nz);
    forward(w, A);
    std::memcpy(out, A.out.data(), sizeof(double) * A.out.size());
}

// training loss over interior cells and its gradient with respect to w; kind 0: mean squared
// error; kind 1: energy norm Σ_p Σ_d c[p,d] (δ[p] - δ[p-e_d])² / n, δ = out - tgt, with c the
// input channels 1..3 (zero in the halo, where δ is zero too)
double orc_nn_loss_grad_kind(const double* w, const double* x0, const double* tgt, int B, int nx, int ny, int nz,
                             int kind, double* grad) {
    Acts A = make(x0, B, nx, ny, nz);
    forward(w, A);
    const Dm &f = A.f, &hf = A.hf, &qt = A.qt;
    const double n = double(B) * nx * ny * nz;
    double loss = 0.0;
    V dout = zeros(f, 1);
    if (kind == 0) {
        FOR_INTERIOR(f) {
            const long long p = f.pos(b, x, y, z);
            const double e = A.out[p] - tgt[p];
            loss += e * e;
            dout[p] = 2.0 * e / n;
        }
    } else {
        V dl = zeros(f, 1);
        for (long long p = 0; p < f.padded(); ++p) dl[p] = A.out[p] - tgt[p];
        const long long off[3] = {1, (long long)(nx + 2), (long long)(nx + 2) * (ny + 2)};
        FOR_INTERIOR(f) {
            const long long p = f.pos(b, x, y, z);
            for (int k = 0; k < 3; ++k) {
                const double c = x0[p * 4 + 1 + k];
                const double jump = dl[p] - dl[p - off[k]];
                loss += c * jump * jump;
                // the face term touches p and p - e_d; the halo cell p - e_d is not an output
                dout[p] += 2.0 * c * jump / n;
                dout[p - off[k]] -= 2.0 * c * jump / n;
            }
        }
        // gradients scattered into halo positions are not outputs of the net
        V keep = zeros(f, 1);
        FOR_INTERIOR(f) {
            const long long p = f.pos(b, x, y, z);
            keep[p] = dout[p];
        }
        dout = keep;
    }
    loss /= n;
    if (!grad) return loss;
    std::memset(grad, 0, sizeof(double) * woff(NL));
    V da5 = zeros(f, 16), dz5 = zeros(f, 16), du1 = zeros(f, 32), da4 = zeros(hf, 32), dz4 = zeros(hf, 32),
      du2 = zeros(hf, 32), da3 = zeros(qt, 32), dz3 = zeros(qt, 32), dp2 = zeros(qt, 32), dz2 = zeros(hf, 32),
      dp1 = zeros(hf, 16), dz1 = zeros(f, 16);
    conv_bwd(f, 16, 1, A.a5, dout, w + woff(5), grad + woff(5), grad + boff(5), &da5);
    relu_bwd(f, 16, A.z5, da5, dz5);
    conv_bwd(f, 32, 16, A.u1, dz5, w + woff(4), grad + woff(4), grad + boff(4), &du1);
    up_bwd(hf, 32, du1, da4);
    relu_bwd(hf, 32, A.z4, da4, dz4);
    conv_bwd(hf, 32, 32, A.u2, dz4, w + woff(3), grad + woff(3), grad + boff(3), &du2);
    up_bwd(qt, 32, du2, da3);
    relu_bwd(qt, 32, A.z3, da3, dz3);
    conv_bwd(qt, 32, 32, A.p2, dz3, w + woff(2), grad + woff(2), grad + boff(2), &dp2);
    V da2 = du2;
    pool_bwd_add(hf, 32, dp2, da2);
    relu_bwd(hf, 32, A.z2, da2, dz2);
    conv_bwd(hf, 16, 32, A.p1, dz2, w + woff(1), grad + woff(1), grad + boff(1), &dp1);
    V da1 = da5;
    pool_bwd_add(f, 16, dp1, da1);
    relu_bwd(f, 16, A.z1, da1, dz1);
    conv_bwd(f, 4, 16, A.x0, dz1, w + woff(0), grad + woff(0), grad + boff(0), nullptr);
    return loss;
}

double orc_nn_loss_grad(const double* w, const double* x0, const double* tgt, int B, int nx, int ny, int nz,
                        double* grad) {
    return orc_nn_loss_grad_kind(w, x0, tgt, B, nx, ny, nz, 0, grad);
}

// one Adam step (β1, β2, ε as the GPU kernel), t = step number starting at 1
void orc_nn_adam(int64_t n, double* w, const double* g, double* m, double* v, double lr, int64_t t) {
    const double b1 = 0.9, b2 = 0.999, eps = 1e-8;
    double c1 = 1.0, c2 = 1.0;
    for (int64_t k = 0; k < t; ++k) {
        c1 *= b1;
        c2 *= b2;
    }
    c1 = 1.0 - c1;
    c2 = 1.0 - c2;
    for (int64_t i = 0; i < n; ++i) {
        m[i] = b1 * m[i] + (1.0 - b1) * g[i];
        v[i] = b2 * v[i] + (1.0 - b2) * g[i] * g[i];
        w[i] -= lr * (m[i] / c1) / (std::sqrt(v[i] / c2) + eps);
    }
}

}  // extern "C"
