// pg_gemm_limb.cu — placeholder for the limb tensor-core form.
#include "pg_common.cuh"

namespace pg {
int limb_rss_matmul_u64(Ctx *c, const uint64_t *const *, const uint64_t *const *, uint64_t *const *,
                        const uint64_t *const *, int, int, int, int, int, int, int) {
    return set_error(c, PG_ERR_UNSUPPORTED, "limb tensor-core form not built");
}
int limb_rss_conv_u64(Ctx *c, const uint64_t *const *, const uint64_t *const *, uint64_t *const *, int, int, int, int,
                      int, int, int, int, int, int) {
    return set_error(c, PG_ERR_UNSUPPORTED, "limb tensor-core form not built");
}
}  // namespace pg
