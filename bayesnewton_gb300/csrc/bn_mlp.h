// Site expectations by the learned surrogate (defined in bn_mlp.cu), called by
// the model engine between the smoother and the site tail.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/bnx.h"

namespace bn {
template <typename T>
struct LikParams;

// For each of the n two-latent sites, (E, g1, g2, h11, h12, h22) of
// E_q log p(y | f) at the marginal (pm [n][2], pv [n][2][2]) into ext [n][6]: the
// network's prediction, or the cubature of lp where -h11 or -h22 is not positive
// (counters[0]) or where a spot-checked site (index % spot == 0) misses the
// cubature by more than tol (counters[1]).  lists: 2 (n + 1) unsigned of scratch.
int mlp_site_expectations(bn_mlp* h, cudaStream_t st, int64_t n, const float* pm, const float* pv, const float* y,
                          const LikParams<float>& lp, int spot, float tol, float* ext, unsigned* counters,
                          unsigned* lists);
}  // namespace bn
