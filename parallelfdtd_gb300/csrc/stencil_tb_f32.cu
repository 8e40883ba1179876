// Temporally blocked update for float field storage.
#include "stencil_tb.cuh"

namespace pfdtd {
int launch_tb_f32(pfdtd_domain* d, void* rec_out, int64_t rec_ld, int64_t inject_end,
                 cudaStream_t s) {
  return tb::launch_tb_p<float>(d, rec_out, rec_ld, inject_end, s);
}
}  // namespace pfdtd
