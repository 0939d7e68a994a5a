// conv_bf16.cu -- tensor-core (tcgen05) convolution; see the kernel file header.
#include "runtime.h"

namespace geye {

geye_status run_conv_bf16(geye_ctx *ctx, Plan &P, ModelPlan &mp) {
  (void)ctx; (void)P; (void)mp;
  set_error("BF16 convolution is not built yet");
  return GEYE_ERR_UNSUPPORTED;
}

}  // namespace geye
