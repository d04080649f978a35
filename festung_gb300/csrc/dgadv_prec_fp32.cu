// Kernels and launch sequences of the FP32 path (stored reals: float), every degree, with the adjoint kernels, the persistent step, the transport kernels and the linked step.
#include "dgadv_device.cuh"

namespace dgadv {
DGADV_DEFINE_TABLES(float, cTf)
}  // namespace dgadv

#include "dgadv_launch.cuh"
#include "dgadv_adjoint.cuh"
#include "dgadv_persist.cuh"
#include "dgadv_transport.cuh"
#include "dgadv_linked.cuh"

namespace dgadv {
const PrecOps &ops_fp32() {
  static const PrecOps ops =
      with_linked<float>(with_transport<float, 0xF>(with_persistent<float, 0xF>(with_adjoint<float, 0xF>(make_ops<float, 0xF, true>()))));
  return ops;
}
}  // namespace dgadv
