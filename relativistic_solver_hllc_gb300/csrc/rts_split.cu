// rts_split.cu -- split-precision tensor-core path (tcgen05).  Placeholder
// until the tcgen05 kernel lands: every entry reports RTS_ERR_UNSUPPORTED.
#include "rts_internal.h"

int rts_split_setup(rts_ctx* ctx, int precision)
{
    return rts_fail(ctx, RTS_ERR_UNSUPPORTED, "precision %d not built yet", precision);
}
int rts_split_step(rts_ctx* ctx, bool, cudaStream_t)
{
    return rts_fail(ctx, RTS_ERR_UNSUPPORTED, "tensor path not built yet");
}
int rts_split_oneshot(rts_ctx* ctx, int, const double*, double, cudaStream_t)
{
    return rts_fail(ctx, RTS_ERR_UNSUPPORTED, "tensor path not built yet");
}
int rts_split_read(rts_ctx* ctx, double*)
{
    return rts_fail(ctx, RTS_ERR_UNSUPPORTED, "tensor path not built yet");
}
int rts_split_read_ibar(rts_ctx* ctx, double*)
{
    return rts_fail(ctx, RTS_ERR_UNSUPPORTED, "tensor path not built yet");
}
void rts_split_free(rts_ctx*) {}
