// pending.cu -- entry points whose implementation lands in later files.
#include "capi_internal.h"

using namespace gg;

namespace gg {
int upload_compressed(genie_index *, const std::vector<uint32_t> &, const std::vector<int64_t> &,
                      const std::vector<int64_t> &, const std::vector<uint32_t> &, const std::vector<uint32_t> &) {
    return fail(GENIE_ERR_NOT_IMPLEMENTED, "compressed indexes are not available in this build");
}
}  // namespace gg

extern "C" {
int genie_index_create_compressed(const int32_t *, int64_t, int32_t, int32_t, int32_t, genie_index **out) {
    if (out) *out = nullptr;
    return fail(GENIE_ERR_NOT_IMPLEMENTED, "compressed indexes are not available in this build");
}
int genie_index_copy_compressed(const genie_index *, uint32_t *, int64_t *, int64_t *, uint32_t *, uint32_t *) {
    return fail(GENIE_ERR_NOT_IMPLEMENTED, "compressed indexes are not available in this build");
}
int64_t genie_codec_encode(int32_t, const uint32_t *, int64_t, uint32_t *, int64_t) { return -GENIE_ERR_NOT_IMPLEMENTED; }
int64_t genie_codec_encode_bound(int64_t n) { return (5 * n) / 4 + 96; }
int genie_codec_decode_device(int32_t, const uint32_t *, const int64_t *, int64_t, const int64_t *, uint32_t *,
                              uint32_t *, void *) {
    return fail(GENIE_ERR_NOT_IMPLEMENTED, "codecs are not available in this build");
}
}
