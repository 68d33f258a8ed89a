// lsdo_params.cpp -- CPU ORACLE (test infrastructure only): the default tuning table, restated
// independently of the product library so that a test can check the two agree byte for byte.
// Meaning of every field: include/lsdg.h.  The values are this project's own (the upstream
// lsd-slam constants are not available: fips.yml:2-4 names an unvendored, unpinned import).
#include <cstring>

#include "lsdo.h"

namespace lsdo {

void default_params(lsdg_params* p) {
  std::memset(p, 0, sizeof(*p));
  p->levels = 5;
  const int iters[LSDG_MAX_LEVELS] = {6, 8, 10, 12, 16, 16};
  for (int i = 0; i < LSDG_MAX_LEVELS; ++i) p->max_iterations[i] = iters[i];
  p->photometric_variance = 16.0f;
  p->huber_delta = 2.0f;
  p->min_z = 0.01f;
  p->border_margin = 2.5f;
  p->lm_lambda_initial = 0.01f;
  p->lm_lambda_up = 4.0f;
  p->lm_lambda_down = 0.5f;
  p->step_eps = 1e-5f;
  p->stall_eps = 5e-4f;
  p->min_good_ratio = 0.5f;
  p->min_usage = 0.2f;
  p->sim3_depth_variance = 1e-4f;
  p->sim3_depth_weight = 1.0f;

  p->min_grad = 5.0f;
  p->min_idepth = 0.05f;
  p->max_idepth = 2.0f;
  p->epipolar_var = 0.25f;
  p->image_var = 4.0f;
  p->min_grad_along_epl2 = 0.1f;
  p->max_ssd = 100.0f;
  p->unique_ratio = 1.2f;
  p->search_sigmas = 2.0f;
  p->max_search_len = 120.0f;
  p->min_search_len = 3.0f;
  p->fuse_chi2 = 6.25f;
  p->min_epl_length = 1.0f;
  p->validity_init = 2;
  p->validity_max = 20;
  p->validity_penalty = 2;
  p->blacklist_limit = 5;

  p->prediction_var = 1e-4f;
  p->propagate_max_photo_diff = 30.0f;

  p->reg_radius = 2;
  p->reg_chi2 = 4.0f;
  p->reg_min_support = 2;
  p->fill_min_support = 8;
  p->fill_var_factor = 2.0f;
  p->refine_prior_weight = 1.0f;
}

}  // namespace lsdo
