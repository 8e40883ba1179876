// Temporally blocked update for __nv_bfloat16 field storage.
#include "stencil_tb.cuh"

namespace pfdtd {
int launch_tb_bf16(pfdtd_domain* d, void* rec_out, int64_t rec_ld, int64_t inject_end,
                  cudaStream_t s) {
  return tb::launch_tb_p<__nv_bfloat16>(d, rec_out, rec_ld, inject_end, s);
}
}  // namespace pfdtd
