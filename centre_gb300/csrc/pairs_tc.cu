// pairs_tc.cu -- joint counts as an FP8 one-hot contraction on tcgen05.
#include "common.cuh"
#include "entropy.cuh"

namespace centre {

bool tc_supported(centre_ctx *ctx, int nb, uint64_t nframes) {
  (void)ctx; (void)nb; (void)nframes;
  return false;
}

int launch_pairs_tc(centre_ctx *ctx, const PairParams &P, const U128 *d_tab, U128 *d_sclnc,
                    unsigned *d_nnz) {
  (void)P; (void)d_tab; (void)d_sclnc; (void)d_nnz;
  return set_error(ctx, CENTRE_E_UNSUPPORTED, "tensor-core counts not available");
}

}  // namespace centre
