// Pass kernels of the 128^3 grid: default configuration first, then autotuner candidates.
#include "ops.cuh"

namespace mhdgb {

OpsBase* make_ops_128() {
  auto* o = new Ops<128>();
  o->add_col<Plan<128, 8, 16, 8>, 16, 2>();
  o->add_col<Plan<128, 8, 16, 8>, 8, 4>();
  o->add_col<Plan<128, 16, 8, 4, 4>, 8, 3>();
  o->add_col_tma<Plan<128, 8, 16, 8>, 2, 2>();
  o->add_x<Plan<128, 16, 8, 4, 4>, 4, 1, 1, 4>();
  o->add_x<Plan<128, 16, 8, 4, 4>, 4, 3, 1, 3>();
  o->add_x<Plan<128, 8, 16, 8>, 4, 1, 1, 2>();
  o->add_x_vp<Plan<128, 16, 8, 4, 4>, 4, 1, 3>();
  o->add_x_hd<Plan<128, 16, 8, 4, 4>, 4, 4>();
  o->add_x_hdvp<Plan<128, 16, 8, 4, 4>, 4, 3>();
  o->add_x_tc<SPLIT_F16, 4, 2>();
  o->add_x_tc<SPLIT_BF16, 4, 2>();
  o->set_rows<Plan<128, 16, 8, 4, 4>, 8>();
  return o;
}

}  // namespace mhdgb
