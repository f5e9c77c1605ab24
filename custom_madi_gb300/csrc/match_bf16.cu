// BF16 tensor-core library match (tcgen05): placeholder until the kernel lands.
#include "madi_device.cuh"
#include "madi_host.h"

using namespace madi;

int64_t madi_match_bf16_scratch(int64_t n_vox, int32_t n_lib, int32_t n_feat, int32_t topk) {
    (void)n_vox; (void)n_lib; (void)n_feat; (void)topk;
    return 0;
}

madi_status madi_match_bf16(const madi_match_desc* d, cudaStream_t s) {
    (void)d; (void)s;
    return host::fail(MADI_ERR_UNSUPPORTED, "match: BF16 path not built");
}
