// Kernels and launch sequences of the FP64 path (stored reals: double), every degree, with the adjoint kernels, the persistent step, the transport kernels and the linked step.
#include "dgadv_device.cuh"

namespace dgadv {
DGADV_DEFINE_TABLES(double, cTd)
}  // namespace dgadv

#include "dgadv_launch.cuh"
#include "dgadv_adjoint.cuh"
#include "dgadv_persist.cuh"
#include "dgadv_transport.cuh"
#include "dgadv_linked.cuh"

namespace dgadv {
const PrecOps &ops_fp64() {
  static const PrecOps ops =
      with_linked<double>(with_transport<double, 0xF>(with_persistent<double, 0xF>(with_adjoint<double, 0xF>(make_ops<double, 0xF, true>()))));
  return ops;
}
}  // namespace dgadv
