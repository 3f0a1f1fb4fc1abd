// unet.cu -- learned warm start for the pressure-correction solve.
// (The implicit-GEMM tcgen05 convolutions land in this file.)

#include "context.cuh"

namespace saras {

int unet_create(Ctx &c) { (void)c; return SARAS_OK; }
void unet_free(Ctx &c) { (void)c; }
int unet_collect(Ctx &c) { c.err = "U-Net warm start not available in this build"; return SARAS_BAD_CONFIG; }
int unet_train(Ctx &c, int iters, double lr, double *loss) {
    (void)iters; (void)lr; (void)loss;
    c.err = "U-Net warm start not available in this build";
    return SARAS_BAD_CONFIG;
}
int unet_infer(Ctx &c, double *out) {
    (void)out;
    c.err = "U-Net warm start not available in this build";
    return SARAS_BAD_CONFIG;
}

}  // namespace saras
