// Instantiates the raymarch kernel for MT_STORAGE_U8 volumes (see mt_march.cuh).
#include "mt_march.cuh"

namespace mt {
cudaError_t launch_march_u8(const MarchArgs& a, cudaStream_t s, long long rays) {
    return launch_march_storage<MT_STORAGE_U8>(a, s, rays);
}
}  // namespace mt
