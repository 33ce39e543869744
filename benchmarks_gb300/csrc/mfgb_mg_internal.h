// mfgb_mg_internal.h -- multigrid level structures shared by the
// single-problem hierarchy (mfgb_mg.cu) and the batched solver (mfgb_batch.cu).
#pragma once
#include <vector>

#include "mfgb_internal.h"

namespace mfgb {

struct MgLevel {
  mfgb_box_desc box{};
  BoxStride bs{};  // s = 1 on the fine mesh (p-levels), 2^l on the l-th h-level
  mfgb_operator *op = nullptr;
  int64_t n = 0;
  void *x = nullptr, *b = nullptr, *r = nullptr, *d = nullptr, *t = nullptr;
  void *inv_diag = nullptr;  // Jacobi (precision T)
  void *inv_val = nullptr;   // 1/valence (precision T), for p-restriction from this level
  double lmax = 0;
  int to_coarse = 0;  // 1 = p-transfer, 2 = h-transfer, 0 = coarsest
  bool borrowed = false;  // op belongs to the caller (mfgb_mg_setup_shared)
};

struct MgCoarse {
  int n = 0;
  double *A = nullptr, *dinv = nullptr, *work = nullptr;
  int64_t *ids = nullptr;
};

// cudaMalloc with a library status
mfgb_status dalloc(void **p, size_t bytes);
// the operator's geometric factors in FP32 (the V-cycle's operator)
mfgb_status ensure_g32(mfgb_operator *op);
// level plan of a fine box: p-levels p, p/2, ..., 1 on the fine mesh, then
// Q1 h-levels of stride 2, 4, ... while the largest cell count exceeds
// coarse_cells; kinds[l] = 1 (p-transfer to l+1), 2 (h-transfer), 0 (coarsest)
void mg_plan_levels(const mfgb_box_desc &fine, int coarse_cells, std::vector<mfgb_box_desc> &boxes,
                    std::vector<int> &kinds, std::vector<int> &strides);
// mfgb_mg_setup without the lambda_max power iterations (every level's lmax
// stays 0): the batched set-up runs them for all its problems at once
mfgb_status mg_setup_without_lmax(const mfgb_box_desc *fine, const mfgb_mg_params *prm,
                                  mfgb_mg **out);

}  // namespace mfgb

struct mfgb_mg {
  int precision = 32;
  int degree = 5;
  double range = 15.0;
  double coarse_tol = 1e-12;
  std::vector<mfgb::MgLevel> levels;
  mfgb::MgCoarse coarse;
  // outer PCG buffers (FP64)
  double *r = nullptr, *z = nullptr, *p = nullptr, *v = nullptr, *part = nullptr,
         *scal = nullptr;
  int64_t outer_n = 0;
};
