// Instantiates the raymarch kernel for MT_STORAGE_BF16 volumes (see mt_march.cuh).
#include "mt_march.cuh"

namespace mt {
cudaError_t launch_march_bf16(const MarchArgs& a, cudaStream_t s, long long rays) {
    return launch_march_storage<MT_STORAGE_BF16>(a, s, rays);
}
cudaError_t launch_batch_bf16(const BatchArgs& b, int lanes, int blocks, cudaStream_t s) {
    return launch_batch_storage<MT_STORAGE_BF16>(b, lanes, blocks, s);
}
int batch_blocks_bf16(int device, int lanes) { return batch_blocks_storage<MT_STORAGE_BF16>(device, lanes); }
}  // namespace mt
