// Pass kernels of the small grid sizes (16, 32, 48, 64, 96): one configuration each.
#include "ops.cuh"

namespace mhdgb {

OpsBase* make_ops_16() {
  auto* o = new Ops<16>();
  o->add_col<Plan<16, 4, 4, 4>, 16, 2>();
  o->add_x<Plan<16, 4, 4, 4>, 4, 1, 1, 4>();
  o->add_x_vp<Plan<16, 4, 4, 4>, 4, 1, 4>();
  o->add_x_hd<Plan<16, 4, 4, 4>, 4, 4>();
  o->add_x_hdvp<Plan<16, 4, 4, 4>, 4, 4>();
  o->set_rows<Plan<16, 4, 4, 4>, 32>();
  return o;
}

OpsBase* make_ops_32() {
  auto* o = new Ops<32>();
  o->add_col<Plan<32, 4, 8, 4>, 16, 2>();
  o->add_col<Plan<32, 4, 8, 4>, 8, 4>();
  o->add_x<Plan<32, 4, 8, 4>, 4, 1, 1, 4>();
  o->add_x_vp<Plan<32, 4, 8, 4>, 4, 1, 4>();
  o->add_x_hd<Plan<32, 4, 8, 4>, 4, 4>();
  o->add_x_hdvp<Plan<32, 4, 8, 4>, 4, 4>();
  o->set_rows<Plan<32, 4, 8, 4>, 32>();
  return o;
}

OpsBase* make_ops_48() {
  auto* o = new Ops<48>();
  o->add_col<Plan<48, 4, 12, 4>, 16, 2>();
  o->add_col<Plan<48, 4, 12, 4>, 8, 4>();
  o->add_x<Plan<48, 4, 12, 4>, 4, 1, 1, 2>();
  o->add_x_vp<Plan<48, 4, 12, 4>, 4, 1, 2>();
  o->add_x_hd<Plan<48, 4, 12, 4>, 4, 2>();
  o->add_x_hdvp<Plan<48, 4, 12, 4>, 4, 2>();
  o->set_rows<Plan<48, 4, 12, 4>, 32>();
  return o;
}

OpsBase* make_ops_64() {
  auto* o = new Ops<64>();
  o->add_col<Plan<64, 8, 8, 8>, 16, 2>();
  o->add_col<Plan<64, 8, 8, 8>, 8, 4>();
  o->add_x<Plan<64, 8, 8, 8>, 4, 1, 1, 4>();
  o->add_x_vp<Plan<64, 8, 8, 8>, 4, 1, 3>();
  o->add_x_hd<Plan<64, 8, 8, 8>, 4, 4>();
  o->add_x_hdvp<Plan<64, 8, 8, 8>, 4, 3>();
  o->set_rows<Plan<64, 8, 8, 8>, 16>();
  return o;
}

OpsBase* make_ops_96() {
  auto* o = new Ops<96>();
  o->add_col<Plan<96, 8, 12, 4, 2>, 16, 2>();
  o->add_col<Plan<96, 8, 12, 4, 2>, 8, 4>();
  o->add_col<Plan<96, 4, 8, 12>, 32, 4>();
  o->add_col<Plan<96, 4, 8, 12>, 16, 8>();
  o->add_x<Plan<96, 8, 12, 4, 2>, 4, 1, 1, 2>();
  o->add_x_vp<Plan<96, 8, 12, 4, 2>, 4, 1, 2>();
  o->add_x_hd<Plan<96, 8, 12, 4, 2>, 4, 2>();
  o->add_x_hdvp<Plan<96, 8, 12, 4, 2>, 4, 2>();
  o->set_rows<Plan<96, 8, 12, 4, 2>, 16>();
  return o;
}

}  // namespace mhdgb
