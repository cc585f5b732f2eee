// Batched replicas (placeholder until the batched engine lands in this file).
#include "common.cuh"
#include "engine.cuh"

using namespace gbmd;

struct gbmd_batch {
    int unused;
};

extern "C" {
int gbmd_batch_create(const gbmd_system*, uint32_t, const uint32_t*, const int64_t*, const int32_t*, const uint32_t*, const gbmd_options*,
                      gbmd_batch** out) {
    if (out) *out = nullptr;
    return fail(GBMD_E_UNSUPPORTED, "batched replicas are not built yet");
}
int gbmd_batch_step(gbmd_batch*, uint64_t) { return fail(GBMD_E_UNSUPPORTED, "batched replicas are not built yet"); }
int gbmd_batch_sync(gbmd_batch*) { return fail(GBMD_E_UNSUPPORTED, "batched replicas are not built yet"); }
int gbmd_batch_read_system(gbmd_batch*, uint32_t, int64_t*, int32_t*, uint32_t*) {
    return fail(GBMD_E_UNSUPPORTED, "batched replicas are not built yet");
}
int gbmd_batch_stream(gbmd_batch*, void**) { return fail(GBMD_E_UNSUPPORTED, "batched replicas are not built yet"); }
int gbmd_batch_destroy(gbmd_batch*) { return GBMD_OK; }
}
