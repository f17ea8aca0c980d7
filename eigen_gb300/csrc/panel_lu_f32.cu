// Panel LU instantiation for float.
#include "panel_lu_impl.cuh"

namespace gbs {
template int panel_factor<float>(cudaStream_t, float*, int64_t, int, int, int, int*, DevBuf&, DeviceStatus*,
                                  const int**, int, bool*, bool);
template int panel_preload<float>();

int panel_cluster_ctas(int m)
{
  int c = 1;
  while (c * kClusterPanelThreads < m && c < kMaxPanelCluster) c *= 2;
  return c;
}
}  // namespace gbs
