// Temporally blocked update, host side: the geometry condition, the
// conditions under which a domain runs blocked, and the dispatch to the
// per-storage-type instantiations (stencil_tb.cuh).
#include "common.cuh"

#include <string>

namespace pfdtd {
int launch_tb_f32(pfdtd_domain* d, void* rec_out, int64_t rec_ld, int64_t inject_end,
                  cudaStream_t s);
int launch_tb_f16(pfdtd_domain* d, void* rec_out, int64_t rec_ld, int64_t inject_end,
                  cudaStream_t s);
int launch_tb_bf16(pfdtd_domain* d, void* rec_out, int64_t rec_ld, int64_t inject_end,
                   cudaStream_t s);

namespace {

constexpr int kMaxSrc = 64;   // list capacities of the blocked kernel
constexpr int kMaxRec = 256;

// Count of updated x/y face nodes whose position byte has the inside bit.
__global__ void k_face_inside(const uint8_t* __restrict__ pos, int X, int Y, int Z,
                              unsigned long long* __restrict__ count) {
  const int64_t per_plane = 2 * (int64_t)X + 2 * (int64_t)Y;
  const int64_t n = per_plane * (Z - 2);
  unsigned long long c = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int z = 1 + (int)(i / per_plane);
    const int64_t r = i % per_plane;
    int x, y;
    if (r < X) { x = (int)r; y = 0; }
    else if (r < 2 * X) { x = (int)(r - X); y = Y - 1; }
    else if (r < 2 * X + Y) { x = 0; y = (int)(r - 2 * X); }
    else { x = X - 1; y = (int)(r - 2 * X - Y); }
    c += (pos[((int64_t)z * Y + y) * X + x] & 0x80u) != 0;
  }
  if (c) atomicAdd(count, c);
}

}  // namespace

int check_tb_faces(pfdtd_domain* d) {
  d->tb_faces_ok = 0;
  if (d->Z < 3) return PFDTD_OK;
  unsigned long long* dc = nullptr;
  cudaStream_t s = d->stream;
  PFDTD_CK(cudaMallocAsync((void**)&dc, sizeof(unsigned long long), s));
  PFDTD_CK(cudaMemsetAsync(dc, 0, sizeof(unsigned long long), s));
  k_face_inside<<<kGridSMs, 256, 0, s>>>(d->d_pos, (int)d->X, (int)d->Y, (int)d->Z, dc);
  count_launch();
  PFDTD_CK(cudaGetLastError());
  unsigned long long h = 1;
  PFDTD_CK(cudaMemcpyAsync(&h, dc, sizeof(h), cudaMemcpyDeviceToHost, s));
  PFDTD_CK(cudaFreeAsync(dc, s));
  PFDTD_CK(cudaStreamSynchronize(s));
  d->tb_faces_ok = h == 0 ? 1 : 0;
  return PFDTD_OK;
}

// Whether the temporally blocked kernel can run this domain as set up; the
// reason when it cannot.
int tb_usable(const pfdtd_domain* d, std::string* why) {
  auto no = [&](const char* w) {
    if (why) *why = w;
    return 0;
  };
  if (d->tb_depth < 2) return no("temporal blocking off");
  if (d->precision == PFDTD_F64) return no("FP64 fields are compute-bound; not blocked");
  if (d->class_scheme != PFDTD_SRL_FORWARD && d->class_scheme != PFDTD_SRL)
    return no("only the SRL forward and centred schemes are blocked");
  if (d->n_dif > 0) return no("frequency-dependent boundaries need the per-step update");
  if (d->class_form != PFDTD_FORM_REFERENCE) return no("the difference form runs the per-step update");
  if (d->cls_bytes != 1) return no("more than 256 node classes");
  if (d->X % 4 != 0) return no("X must be a multiple of 4");
  if (d->K != 1 && d->K % 4 != 0) return no("batched fields must be a multiple of 4");
  if (d->Z < 3) return no("fewer than 3 planes");
  if (!d->tb_faces_ok) return no("an x/y face node is inside the room (flat-index wrap)");
  if (d->n_src > kMaxSrc) return no("more than 64 sources");
  if (d->n_rec > kMaxRec) return no("more than 256 receivers");
  if (d->X * d->Y * d->Z >= ((int64_t)1 << 40)) return no("grid too large");
  for (int64_t e : d->src_idx_h) {
    if (e < 0) continue;
    const int64_t z = (e >> d->kshift) / d->XY;
    if (z == 0 || z == d->Z - 1) return no("a source lies on plane 0 or Z-1");
  }
  for (int64_t e : d->rec_idx_h) {
    if (e < 0) continue;
    const int64_t z = (e >> d->kshift) / d->XY;
    if (z == 0 || z == d->Z - 1) return no("a receiver lies on plane 0 or Z-1");
  }
  if (!d->field_base[2] || !d->field_base[3]) return no("blocking buffers not allocated");
  return 1;
}

int launch_tb(pfdtd_domain* d, void* rec_out, int64_t rec_ld, int64_t inject_end,
              cudaStream_t s) {
  int rc = launch_io(d, d->cur_field(), rec_out, rec_ld, inject_end, s, d->tb_depth);
  if (rc) return rc;
  switch (d->precision) {
    case PFDTD_F32: return launch_tb_f32(d, rec_out, rec_ld, inject_end, s);
    case PFDTD_F16: return launch_tb_f16(d, rec_out, rec_ld, inject_end, s);
    case PFDTD_BF16: return launch_tb_bf16(d, rec_out, rec_ld, inject_end, s);
  }
  return fail(PFDTD_ERR_UNSUPPORTED, "precision not blocked");
}

bool tb_shape_valid(const pfdtd_domain* d, int shape) {
  if (shape < 0) return true;
  if (d->tb_depth == 4) return shape == 1;
  if (d->K > 1 && (shape == 2 || shape == 3))  // packed pair kernel: forward, a free class slot
    return d->class_scheme == PFDTD_SRL_FORWARD && d->n_classes < 256;
  return shape < 3;
}

}  // namespace pfdtd
