// Anomaly-to-anomaly Green tensor build on the device.
#include "egx_green.cuh"

extern "C" int egx_green_build(egx_ctx *ctx, const egx_model *model, double omega, int n_hankels, int precision,
                               egx_green **out) {
    (void)ctx; (void)model; (void)omega; (void)n_hankels; (void)precision;
    if (out) *out = nullptr;
    return EGX_ERR_STATE;
}
