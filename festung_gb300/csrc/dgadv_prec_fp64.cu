// Kernels and launch sequences of the FP64 path (stored reals: double), every degree.
#include "dgadv_device.cuh"

namespace dgadv {
DGADV_DEFINE_TABLES(double, cTd)
}  // namespace dgadv

#include "dgadv_launch.cuh"

namespace dgadv {
const PrecOps &ops_fp64() {
  static const PrecOps ops = make_ops<double, 0xF, true>();
  return ops;
}
}  // namespace dgadv
