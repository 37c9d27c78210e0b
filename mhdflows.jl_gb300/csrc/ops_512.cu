// Pass kernels of the 512^3 grid: default configuration first, then autotuner candidates.
#include "ops.cuh"

namespace mhdgb {

OpsBase* make_ops_512() {
  auto* o = new Ops<512>();
  o->add_col<Plan<512, 32, 16, 8, 4>, 16, 1>();
  o->add_col<Plan<512, 32, 16, 8, 4>, 8, 2>();
  o->add_col<Plan<512, 64, 8, 8, 8>, 8, 1>();
  o->add_col<Plan<512, 32, 16, 8, 4>, 8, 1, 3>();
  o->add_col<Plan<512, 32, 16, 8, 4>, 8, 2, 3>();
  o->add_col_tma<Plan<512, 32, 16, 8, 4>, 1, 2>();
  o->add_col<Plan<512, 32, 16, 8, 4>, 16, 1, 2, true>();
  o->add_col<Plan<512, 32, 16, 8, 4>, 8, 2, 2, true>();
  o->add_col_tma<Plan<512, 32, 16, 8, 4>, 1, 2, true>();
  o->add_col<Plan<512, 16, 32, 16>, 16, 1, 2, true>();
  o->add_col<Plan<512, 16, 32, 16>, 16, 1, 3, true>();
  o->add_col_tma<Plan<512, 16, 32, 16>, 1, 2, true>();
  o->add_col_tma<Plan<512, 16, 32, 16>, 1, 3, true>();
  o->add_x<Plan<512, 64, 8, 8, 8>, 2, 1, 1, 4>();
  o->add_x<Plan<512, 32, 16, 8, 4>, 4, 1, 1, 2>();
  o->add_x<Plan<512, 32, 8, 8, 8>, 4, 1, 1, 2>();
  o->add_x_form<Plan<512, 32, 8, 8, 8>, 4, 1, 1, 2, true>();
  o->add_x_vp<Plan<512, 64, 8, 8, 8>, 2, 1, 4>();
  o->add_x_hd<Plan<512, 64, 8, 8, 8>, 2, 4>();
  o->add_x_hdvp<Plan<512, 64, 8, 8, 8>, 2, 4>();
  o->add_x_tc<SPLIT_F16, 4, 2>();
  o->add_x_tc<SPLIT_BF16, 4, 2>();
  o->set_rows<Plan<512, 64, 8, 8, 8>, 2>();
  return o;
}

}  // namespace mhdgb
