#include "mz_host.h"
void launch_merge(mz_domain*, int, int64_t, int64_t, int64_t, int64_t, const mz_octree_params*, const mz_grid1d*,
                  uint64_t, int64_t*)
{
    throw MzError(MZ_E_ARG, "octree merge not built");
}
