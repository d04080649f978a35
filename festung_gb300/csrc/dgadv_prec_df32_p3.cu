// Kernels and launch sequences of the double-float path (stored reals: df32), degree 3.
// The df32 kernels are large (every operation expands to several FP32 instructions), so each
// degree compiles in a unit of its own; the opt-in fused kernels are not built for df32.
#include "dgadv_device.cuh"

namespace dgadv {
DGADV_DEFINE_TABLES(df32, cTw)
}  // namespace dgadv

#include "dgadv_launch.cuh"

namespace dgadv {
const PrecOps &ops_df32_p3() {
  static const PrecOps ops = make_ops<df32, 0x8, false>();
  return ops;
}
}  // namespace dgadv
