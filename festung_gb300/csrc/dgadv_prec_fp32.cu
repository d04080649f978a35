// Kernels and launch sequences of the FP32 path (stored reals: float), every degree.
#include "dgadv_device.cuh"

namespace dgadv {
DGADV_DEFINE_TABLES(float, cTf)
}  // namespace dgadv

#include "dgadv_launch.cuh"

namespace dgadv {
const PrecOps &ops_fp32() {
  static const PrecOps ops = make_ops<float, 0xF, true>();
  return ops;
}
}  // namespace dgadv
