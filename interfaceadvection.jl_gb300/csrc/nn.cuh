// Learned Poisson preconditioner: a 3-level 3D convolutional encoder-decoder
// (16/32/32 channels, 3x3x3 kernels) mapping (normalised residual, face
// coefficients) to a pressure correction, used inside flexible CG with the
// multigrid V-cycle as fallback.  No counterpart in the reference.
//
// Layers (all 3x3x3, stride 1, zero padding; activations channels-last with a
// one-cell zero halo):
//   c1: 4->16  ReLU            full res        a1
//   avg-pool 2                 half res
//   c2: 16->32 ReLU            half            a2
//   avg-pool 2                 quarter
//   c3: 32->32 ReLU            quarter         a3
//   nearest x2, + a2           half            u2
//   c4: 32->32 ReLU            half            a4
//   nearest x2                 full            u1
//   c5: 32->16 ReLU, + a1      full            a5
//   c6: 16->1  (linear)        full            out
// Inputs: r/s, λρ·L_x, λρ·L_y, λρ·L_z with s = max|r|; output × s = correction.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace ia {
namespace nn {

constexpr int NLAYER = 6;
constexpr int CIN[NLAYER] = {4, 16, 32, 32, 32, 16};
constexpr int COUT[NLAYER] = {16, 32, 32, 32, 16, 1};
constexpr int LEVEL[NLAYER] = {0, 1, 2, 1, 0, 0};   // 0 full, 1 half, 2 quarter

// offsets of W_l [27][Cout][Cin] then b_l [Cout] in the FP32 parameter vector
constexpr long long layer_w(int l) {
    long long o = 0;
    for (int k = 0; k < l; ++k) o += 27LL * COUT[k] * CIN[k] + COUT[k];
    return o;
}
constexpr long long layer_b(int l) { return layer_w(l) + 27LL * COUT[l] * CIN[l]; }
constexpr long long NPARAM = layer_w(NLAYER);

}  // namespace nn
}  // namespace ia
