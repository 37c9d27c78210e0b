// Pass kernels of the 256^3 grid: default configuration first, then autotuner candidates.
#include "ops.cuh"

namespace mhdgb {

OpsBase* make_ops_256() {
  auto* o = new Ops<256>();
  o->add_col<Plan<256, 16, 16, 16>, 16, 3>();
  o->add_col<Plan<256, 16, 16, 16>, 8, 4>();
  o->add_col<Plan<256, 32, 8, 8, 4>, 8, 3>();
  o->add_col<Plan<256, 32, 8, 8, 4>, 16, 2>();
  o->add_col<Plan<256, 32, 8, 8, 4>, 16, 3>();
  o->add_col<Plan<256, 16, 16, 16>, 16, 4>();
  o->add_col<Plan<256, 16, 16, 16>, 16, 2, 3>();
  o->add_col<Plan<256, 16, 16, 16>, 8, 4, 4>();
  o->add_col<Plan<256, 16, 16, 16>, 8, 6, 3>();
  o->add_col_tma<Plan<256, 16, 16, 16>, 3, 2>();
  o->add_col_tma<Plan<256, 16, 16, 16>, 2, 3>();
  o->add_x<Plan<256, 32, 8, 8, 4>, 4, 1, 1, 4>();
  o->add_x<Plan<256, 32, 8, 8, 4>, 4, 3, 1, 3>();
  o->add_x<Plan<256, 32, 8, 8, 4>, 4, 3, 2, 3>();
  o->add_x<Plan<256, 16, 16, 16>, 4, 1, 1, 2>();
  o->add_x<Plan<256, 32, 8, 8, 4>, 8, 1, 1, 2>();
  o->add_x<Plan<256, 32, 8, 8, 4>, 2, 1, 1, 8>();
  o->add_x_vp<Plan<256, 32, 8, 8, 4>, 4, 1, 3>();
  o->add_x_hd<Plan<256, 32, 8, 8, 4>, 8, 2>();
  o->add_x_hd<Plan<256, 32, 8, 8, 4>, 4, 4>();
  o->add_x_hdvp<Plan<256, 32, 8, 8, 4>, 4, 3>();
  o->add_x_tc<SPLIT_F16, 4, 2>();
  o->add_x_tc<SPLIT_BF16, 4, 2>();
  o->add_x_tc5();
  o->set_rows<Plan<256, 32, 8, 8, 4>, 4>();
  return o;
}

}  // namespace mhdgb
