// Panel LU instantiation for double.
#include "panel_lu_impl.cuh"

namespace gbs {
template int panel_factor<double>(cudaStream_t, double*, int64_t, int, int, int, int*, DevBuf&, DeviceStatus*,
                                  const int**, int, bool*, bool);
template int panel_preload<double>();
}  // namespace gbs
