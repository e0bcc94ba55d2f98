// Per-point losses of the trainers and their derivative seeds, shared by
// the FP32 loss kernel and the fused tensor-core training kernel.
//
//   MPL_LOSS_RESIDUAL  loss_add_detail / loss_add_detail_fine
//                      (i3d/loss_functions.py:263-394), with S = f + frozen
//                      sums and G = df/dx + frozen sums: terms
//                      [(gt - S)^2, 1 - cos(n, G), (|G| - 1)^2], the first
//                      two where gt != -1;
//   MPL_LOSS_TRUE_SDF  true_sdf (i3d/loss_functions.py:123-163): terms
//                      [S^2 where gt == 0, (gt - S)^2 where gt != 0,
//                      1 - cos(G, n) where gt == 0, (|G| - 1)^2].
// Each term is a mean over all n points times its weight; the seeds are
// dL/dS (phi) and dL/dG (gam).  torch's cosine_similarity clamps each norm
// at 1e-8 separately.
#pragma once

#include "common.cuh"

namespace mpl {

struct LossParams {
  int kind;
  float w[4];
  float inv_n;
};

__device__ __forceinline__ void point_loss(const LossParams& L, float S, const float (&G)[3],
                                           float gt, const float (&N)[3], float& phi,
                                           float (&gam)[3], float (&term)[4]) {
  phi = 0.f;
  gam[0] = gam[1] = gam[2] = 0.f;
  term[0] = term[1] = term[2] = term[3] = 0.f;
  const float gl = sqrtf(G[0] * G[0] + G[1] * G[1] + G[2] * G[2]);
  const bool residual = L.kind == MPL_LOSS_RESIDUAL;
  // where the normal term applies, and its weight and output slot
  const bool normal_on = residual ? gt != -1.0f : gt == 0.0f;
  const float w_normal = residual ? L.w[1] : L.w[2];
  const float w_eik = residual ? L.w[2] : L.w[3];
  if (residual) {
    if (gt != -1.0f) {
      const float r = __fsub_rn(gt, S);
      term[0] = r * r;
      phi = -2.0f * r * L.w[0] * L.inv_n;
    }
  } else if (gt == 0.0f) {
    term[0] = S * S;
    phi = 2.0f * S * L.w[0] * L.inv_n;
  } else {
    const float r = __fsub_rn(gt, S);
    term[1] = r * r;
    phi = -2.0f * r * L.w[1] * L.inv_n;
  }
  if (normal_on) {
    const float nl = sqrtf(N[0] * N[0] + N[1] * N[1] + N[2] * N[2]);
    const float nn = fmaxf(nl, 1e-8f), gg = fmaxf(gl, 1e-8f);
    const float cosv = (N[0] * G[0] + N[1] * G[1] + N[2] * G[2]) / (nn * gg);
    term[residual ? 1 : 2] = 1.0f - cosv;
    // d(1 - cos)/dG = -(N / (nn gg) - cos G / gg^2)  (the second part only when gl > eps)
    const float sc = w_normal * L.inv_n;
    const float cg = gl > 1e-8f ? cosv / (gg * gg) : 0.f;
    for (int c = 0; c < 3; ++c) gam[c] -= sc * (N[c] / (nn * gg) - cg * G[c]);
  }
  const float ge = gl - 1.0f;
  term[residual ? 2 : 3] = ge * ge;
  if (gl > 0.f) {
    const float sc = 2.0f * ge * w_eik * L.inv_n / gl;
    for (int c = 0; c < 3; ++c) gam[c] += sc * G[c];
  }
}

__host__ inline int loss_params(const MplLoss* loss, int64_t n, LossParams* L) {
  if (!loss || (loss->kind != MPL_LOSS_RESIDUAL && loss->kind != MPL_LOSS_TRUE_SDF))
    return MPL_ERR_INVALID_ARG;
  L->kind = loss->kind;
  for (int i = 0; i < 4; ++i) L->w[i] = loss->weight[i];
  L->inv_n = n > 0 ? 1.0f / (float)n : 0.f;
  return MPL_OK;
}

}  // namespace mpl
