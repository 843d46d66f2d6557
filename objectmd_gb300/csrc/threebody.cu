// Three-body kernels (Stillinger-Weber, Tersoff) and the ZBL pair.
#include "device_common.cuh"

namespace omdg {

int threebody_prepare(Context* c) { return OMDG_OK; }
int sw_launch(Context* c, Potential&, bool) { return set_error(c, OMDG_EINVAL, "SW not built yet"); }
int tersoff_launch(Context* c, Potential&, bool) { return set_error(c, OMDG_EINVAL, "Tersoff not built yet"); }
int zbl_launch(Context* c, Potential&, bool) { return set_error(c, OMDG_EINVAL, "ZBL not built yet"); }

}  // namespace omdg
