// Instantiates the raymarch kernel for MT_STORAGE_F16 volumes (see mt_march.cuh).
#include "mt_march.cuh"

namespace mt {
cudaError_t launch_march_f16(const MarchArgs& a, cudaStream_t s, long long rays) {
    return launch_march_storage<MT_STORAGE_F16>(a, s, rays);
}
}  // namespace mt
