// Solid voxelization of a triangle mesh into the voxelizer's node bytes.
//
// The reference voxelizes with an external library (hakarlss/Voxelizer,
// not vendored, version unpinned; called from
// src/kernels/voxelizationUtils.cu:55-136) whose output is one boundary id
// 0..27 per node (0 solid, 1..8 corners, 9..20 edges, 21..26 faces, 27 air)
// and one material byte.  This file produces the same two arrays on the GPU
// from the room's boundary mesh (closed; closed obstacles inside):
//
//  * grid: node i at lo + (i - 1) dx per axis, lo the mesh's bounding-box
//    minimum, so that a point p of the mesh maps to node ROUND((p - lo)/dx) + 1
//    as the reference's source and receiver coordinates do
//    (SimulationParameters.cpp:200-224); one layer outside the box on every
//    side, so the outermost nodes are solid.  Nodes are sampled a small
//    irrational fraction of dx above their nominal position on every axis, so
//    a node on a wall plane belongs to the side the offset points to;
//  * solid / air: one thread per (x, y) column casts a ray along +z and counts
//    triangle crossings below each node (odd = inside the room = air); the
//    sampling offset keeps the ray off the shared edges of a grid-aligned
//    mesh; the geometry is evaluated in double;
//  * air nodes with solid on both sides of an axis have no boundary id in the
//    voxelizer's table and are made solid, repeatedly until none is left;
//  * materials: a solid node next to air takes the material of the triangle
//    crossed by the segment to its first air neighbour (order -x, +x, -y, +y,
//    -z, +z); a solid node filled in by the previous rule takes its first
//    solid neighbour's material; a boundary node takes the material of its
//    first solid neighbour in the same order, air nodes 0;
//  * ids from the 6-neighbour missing mask with the voxelizer's table.
// These conventions are the ones of parallelfdtd_gb300/rooms.py, so a
// grid-aligned box mesh voxelizes to exactly the procedural room.
#include "common.cuh"

#include <algorithm>
#include <vector>

namespace pfdtd {
namespace {

constexpr int kMaxCrossings = 64;   // triangle crossings per column
constexpr int kTriTile = 128;       // triangles staged in shared memory per pass
// sampling offsets (fractions of dx) per axis
constexpr double kEpsX = 1.2345678901e-5, kEpsY = 3.1415926536e-5, kEpsZ = 2.2360679775e-5;

// Missing-neighbour mask (bit set = solid) -> boundary id; 0 where a mask has
// both sides of an axis missing (no id in the voxelizer's table).
__constant__ uint8_t c_bid_lut[64] = {
    27, 24, 25, 0, 22, 20, 19, 0, 23, 18, 17, 0, 0, 0, 0, 0, 26, 16, 15, 0, 14, 8,
    7,  0,  13, 6, 5,  0,  0,  0, 0, 0, 21, 12, 11, 0, 10, 4, 3, 0, 9, 2,  1,  0, 0,
    0,  0,  0,  0, 0,  0,  0,  0, 0, 0, 0,  0,  0,  0, 0, 0, 0, 0, 0};

struct Tri {
  float v[9];      // three vertices
  uint32_t mat;    // material byte
};

__device__ __forceinline__ bool valid_mask(unsigned m) {
  return (m & 3u) != 3u && (m & 12u) != 12u && (m & 48u) != 48u;
}

// Crossing of the line {(a0, a1) fixed, t free} with a triangle, the line's
// free axis `ax` and the two fixed axes (c0, c1): returns true and t when the
// point (a0, a1) lies strictly inside the triangle's projection.
__device__ __forceinline__ bool line_cross(const Tri& t, int ax, int c0, int c1, double a0,
                                           double a1, double* tt) {
  const double x0 = t.v[c0], y0 = t.v[c1], x1 = t.v[3 + c0], y1 = t.v[3 + c1];
  const double x2 = t.v[6 + c0], y2 = t.v[6 + c1];
  const double e0 = (x1 - x0) * (a1 - y0) - (y1 - y0) * (a0 - x0);
  const double e1 = (x2 - x1) * (a1 - y1) - (y2 - y1) * (a0 - x1);
  const double e2 = (x0 - x2) * (a1 - y2) - (y0 - y2) * (a0 - x2);
  const bool in = (e0 > 0 && e1 > 0 && e2 > 0) || (e0 < 0 && e1 < 0 && e2 < 0);
  if (!in) return false;
  const double area = e0 + e1 + e2;
  if (area == 0.0) return false;
  // barycentric weights of vertices 2, 0, 1 are e0, e1, e2 over the area
  *tt = (e1 * t.v[ax] + e2 * t.v[3 + ax] + e0 * t.v[6 + ax]) / area;
  return true;
}

// Column parity: solid[] = 1 outside the room, 0 inside.
__global__ void k_parity(const Tri* __restrict__ tris, int64_t nt, int X, int Y, int Z,
                         double lo_x, double lo_y, double lo_z, double dx,
                         uint8_t* __restrict__ solid, int* __restrict__ err) {
  __shared__ Tri st[kTriTile];
  const int64_t col = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const bool active = col < (int64_t)X * Y;
  const int i = active ? (int)(col % X) : 0, j = active ? (int)(col / X) : 0;
  const double px = lo_x + (i - 1 + kEpsX) * dx;
  const double py = lo_y + (j - 1 + kEpsY) * dx;
  double zc[kMaxCrossings];
  int nc = 0;
  bool overflow = false;
  for (int64_t base = 0; base < nt; base += kTriTile) {
    __syncthreads();
    for (int k = threadIdx.x; k < kTriTile && base + k < nt; k += blockDim.x) st[k] = tris[base + k];
    __syncthreads();
    const int n = (int)(nt - base < kTriTile ? nt - base : (int64_t)kTriTile);
    if (!active) continue;
    for (int k = 0; k < n; ++k) {
      double t;
      if (line_cross(st[k], 2, 0, 1, px, py, &t)) {
        if (nc < kMaxCrossings) zc[nc++] = t;
        else overflow = true;
      }
    }
  }
  if (!active) return;
  if (overflow) atomicExch(err, 1);
  // insertion sort of the crossings along z
  for (int a = 1; a < nc; ++a) {
    const double v = zc[a];
    int b = a - 1;
    while (b >= 0 && zc[b] > v) { zc[b + 1] = zc[b]; --b; }
    zc[b + 1] = v;
  }
  int below = 0;
  for (int k = 0; k < Z; ++k) {
    const double z = lo_z + (k - 1 + kEpsZ) * dx;
    while (below < nc && zc[below] < z) ++below;
    solid[((int64_t)k * Y + j) * X + i] = (below & 1) ? 0 : 1;
  }
}

__device__ __forceinline__ int64_t nb_index(int64_t c, int d, int X, int64_t XY) {
  switch (d) {
    case 0: return c - 1;
    case 1: return c + 1;
    case 2: return c - X;
    case 3: return c + X;
    case 4: return c - XY;
    default: return c + XY;
  }
}

__device__ __forceinline__ bool nb_inside(int x, int y, int z, int d, int X, int Y, int Z) {
  switch (d) {
    case 0: return x > 0;
    case 1: return x < X - 1;
    case 2: return y > 0;
    case 3: return y < Y - 1;
    case 4: return z > 0;
    default: return z < Z - 1;
  }
}

// Missing-neighbour mask of node c (neighbours outside the grid count solid).
__device__ __forceinline__ unsigned missing_mask(const uint8_t* __restrict__ solid, int64_t c,
                                                 int x, int y, int z, int X, int Y, int Z,
                                                 int64_t XY) {
  unsigned m = 0;
#pragma unroll
  for (int d = 0; d < 6; ++d)
    if (!nb_inside(x, y, z, d, X, Y, Z) || solid[nb_index(c, d, X, XY)]) m |= 1u << d;
  return m;
}

// Surface materials: a solid node with an air neighbour takes the material
// of the triangle crossed by the segment to its first air neighbour (the
// crossing nearest to the node); 255 when no triangle crosses it.
__global__ void k_surface_mat(const Tri* __restrict__ tris, int64_t nt, const uint8_t* __restrict__ solid,
                              int X, int Y, int Z, double lo_x, double lo_y, double lo_z,
                              double dx, uint8_t* __restrict__ smat) {
  __shared__ Tri st[kTriTile];
  const int64_t XY = (int64_t)X * Y, N = XY * Z;
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int dir = -1;
  int x = 0, y = 0, z = 0;
  if (c < N && solid[c]) {
    x = (int)(c % X);
    y = (int)((c / X) % Y);
    z = (int)(c / XY);
    for (int d = 0; d < 6 && dir < 0; ++d)
      if (nb_inside(x, y, z, d, X, Y, Z) && !solid[nb_index(c, d, X, XY)]) dir = d;
  }
  // blocks without a surface node skip the triangle loop (uniform per block)
  if (!__syncthreads_or(dir >= 0)) return;
  const int ax = dir < 0 ? 0 : dir >> 1;
  const double sgn = (dir & 1) ? 1.0 : -1.0;
  const double p[3] = {lo_x + (x - 1 + kEpsX) * dx, lo_y + (y - 1 + kEpsY) * dx,
                       lo_z + (z - 1 + kEpsZ) * dx};
  const int c0 = ax == 0 ? 1 : 0, c1 = ax == 2 ? 1 : 2;
  double best = 2.0;
  uint32_t best_mat = 255;
  for (int64_t base = 0; base < nt; base += kTriTile) {
    __syncthreads();
    for (int k = threadIdx.x; k < kTriTile && base + k < nt; k += blockDim.x) st[k] = tris[base + k];
    __syncthreads();
    if (dir < 0) continue;
    const int n = (int)(nt - base < kTriTile ? nt - base : (int64_t)kTriTile);
    for (int k = 0; k < n; ++k) {
      double t;
      if (line_cross(st[k], ax, c0, c1, p[c0], p[c1], &t)) {
        const double s = (t - p[ax]) * sgn / dx;  // distance along the segment, in voxels
        if (s >= 0.0 && s <= 1.0 && s < best) {
          best = s;
          best_mat = st[k].mat;
        }
      }
    }
  }
  if (dir >= 0) smat[c] = (uint8_t)best_mat;
}

// One Jacobi pass of the slot closing: air nodes with solid on both sides of
// an axis become solid with their first solid neighbour's material.
__global__ void k_close_slots(const uint8_t* __restrict__ solid, const uint8_t* __restrict__ smat,
                              uint8_t* __restrict__ solid_out, uint8_t* __restrict__ smat_out,
                              int X, int Y, int Z, int* __restrict__ changed) {
  const int64_t XY = (int64_t)X * Y, N = XY * Z;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < N;
       c += (int64_t)gridDim.x * blockDim.x) {
    uint8_t s = solid[c], m = smat[c];
    if (!s) {
      const int x = (int)(c % X), y = (int)((c / X) % Y), z = (int)(c / XY);
      const unsigned mk = missing_mask(solid, c, x, y, z, X, Y, Z, XY);
      if (!valid_mask(mk)) {
        s = 1;
        for (int d = 0; d < 6; ++d)
          if (nb_inside(x, y, z, d, X, Y, Z) && solid[nb_index(c, d, X, XY)]) {
            m = smat[nb_index(c, d, X, XY)];
            break;
          }
        *changed = 1;
      }
    }
    solid_out[c] = s;
    smat_out[c] = m;
  }
}

// Boundary ids and materials.
__global__ void k_ids(const uint8_t* __restrict__ solid, const uint8_t* __restrict__ smat, int X,
                      int Y, int Z, uint8_t* __restrict__ bid, uint8_t* __restrict__ mat) {
  const int64_t XY = (int64_t)X * Y, N = XY * Z;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < N;
       c += (int64_t)gridDim.x * blockDim.x) {
    if (solid[c]) {
      bid[c] = 0;
      mat[c] = 0;
      continue;
    }
    const int x = (int)(c % X), y = (int)((c / X) % Y), z = (int)(c / XY);
    const unsigned mk = missing_mask(solid, c, x, y, z, X, Y, Z, XY);
    const uint8_t b = c_bid_lut[mk];
    bid[c] = b;
    uint8_t m = 0;
    if (b > 0 && b < 27) {
      for (int d = 0; d < 6; ++d)
        if (nb_inside(x, y, z, d, X, Y, Z) && solid[nb_index(c, d, X, XY)]) {
          m = smat[nb_index(c, d, X, XY)];
          break;
        }
      if (m == 255) m = 0;
    }
    mat[c] = m;
  }
}

int grid_n(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, kGridSMs * 32)); }

}  // namespace
}  // namespace pfdtd

using namespace pfdtd;

extern "C" int pfdtd_voxelize(const float* vertices, int64_t n_vertices, const uint32_t* indices,
                              int64_t n_triangles, const uint8_t* tri_materials,
                              double voxel_edge, int device, uint32_t dims[3], double origin[3],
                              uint8_t* bid_out, uint8_t* mat_out) {
  if (!vertices || !indices || n_vertices < 3 || n_triangles < 1 || !dims)
    return fail(PFDTD_ERR_ARG, "invalid mesh");
  if (!(voxel_edge > 0.0)) return fail(PFDTD_ERR_ARG, "voxel edge must be positive");
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int64_t v = 0; v < n_vertices; ++v)
    for (int a = 0; a < 3; ++a) {
      const double c = vertices[3 * v + a];
      if (!(c == c)) return fail(PFDTD_ERR_ARG, "vertex coordinate is NaN");
      lo[a] = std::min(lo[a], c);
      hi[a] = std::max(hi[a], c);
    }
  // last inside node: the largest i with (i - 1 + eps) dx < extent; one
  // outside layer beyond it
  int64_t n[3];
  const double eps[3] = {kEpsX, kEpsY, kEpsZ};
  for (int a = 0; a < 3; ++a) {
    n[a] = (int64_t)std::floor((hi[a] - lo[a]) / voxel_edge - eps[a]) + 3;
    if (n[a] < 3) n[a] = 3;
  }
  if (n[0] > (1 << 20) || n[1] > (1 << 20) || n[2] > (1 << 20) ||
      n[0] * n[1] * n[2] > ((int64_t)1 << 36))
    return fail(PFDTD_ERR_ARG, "voxel grid too large");
  for (int a = 0; a < 3; ++a) dims[a] = (uint32_t)n[a];
  if (origin)
    for (int a = 0; a < 3; ++a) origin[a] = lo[a] - voxel_edge;  // position of node 0
  if (!bid_out && !mat_out) return PFDTD_OK;
  if (!bid_out || !mat_out) return fail(PFDTD_ERR_ARG, "both output arrays are needed");
  std::vector<Tri> tris((size_t)n_triangles);
  for (int64_t t = 0; t < n_triangles; ++t) {
    for (int k = 0; k < 3; ++k) {
      const uint32_t vi = indices[3 * t + k];
      if ((int64_t)vi >= n_vertices) return fail(PFDTD_ERR_ARG, "triangle index out of range");
      for (int a = 0; a < 3; ++a) tris[t].v[3 * k + a] = vertices[3 * (int64_t)vi + a];
    }
    tris[t].mat = tri_materials ? tri_materials[t] : 0;
  }
  const int X = (int)n[0], Y = (int)n[1], Z = (int)n[2];
  const int64_t N = (int64_t)X * Y * Z;
  int prev = -1;
  cudaGetDevice(&prev);
  if (prev != device) cudaSetDevice(device);
  struct Restore {
    int p;
    ~Restore() { if (p >= 0) cudaSetDevice(p); }
  } restore{prev};
  cudaStream_t s = nullptr;
  PFDTD_CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  Tri* d_tris = nullptr;
  uint8_t *d_solid = nullptr, *d_smat = nullptr, *d_s2 = nullptr, *d_m2 = nullptr;
  int* d_flags = nullptr;  // [0] overflow, [1] changed
  cudaError_t e = cudaMallocAsync((void**)&d_tris, sizeof(Tri) * tris.size(), s);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&d_solid, N, s);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&d_smat, N, s);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&d_s2, N, s);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&d_m2, N, s);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&d_flags, 2 * sizeof(int), s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_tris, tris.data(), sizeof(Tri) * tris.size(), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_flags, 0, 2 * sizeof(int), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_smat, 255, N, s);
  int flags[2] = {0, 0};
  if (e == cudaSuccess) {
    const int64_t cols = (int64_t)X * Y;
    k_parity<<<(int)((cols + 127) / 128), 128, 0, s>>>(d_tris, n_triangles, X, Y, Z, lo[0], lo[1],
                                                        lo[2], voxel_edge, d_solid, d_flags);
    count_launch();
    k_surface_mat<<<(int)((N + 127) / 128), 128, 0, s>>>(d_tris, n_triangles, d_solid, X, Y, Z,
                                                          lo[0], lo[1], lo[2], voxel_edge, d_smat);
    count_launch();
    e = cudaGetLastError();
  }
  // close slots until none is left (each pass ping-pongs the two buffers)
  for (int pass = 0; e == cudaSuccess && pass < 4096; ++pass) {
    e = cudaMemsetAsync(d_flags + 1, 0, sizeof(int), s);
    if (e != cudaSuccess) break;
    k_close_slots<<<grid_n(N), 256, 0, s>>>(d_solid, d_smat, d_s2, d_m2, X, Y, Z, d_flags + 1);
    count_launch();
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(flags, d_flags, sizeof(flags), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    std::swap(d_solid, d_s2);
    std::swap(d_smat, d_m2);
    if (e != cudaSuccess || !flags[1]) break;
  }
  if (e == cudaSuccess) {
    k_ids<<<grid_n(N), 256, 0, s>>>(d_solid, d_smat, X, Y, Z, d_s2, d_m2);
    count_launch();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(bid_out, d_s2, N, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(mat_out, d_m2, N, cudaMemcpyDeviceToHost, s);
  for (void* p : {(void*)d_tris, (void*)d_solid, (void*)d_smat, (void*)d_s2, (void*)d_m2,
                  (void*)d_flags})
    if (p) cudaFreeAsync(p, s);
  const cudaError_t e2 = cudaStreamSynchronize(s);
  cudaStreamDestroy(s);
  if (e == cudaSuccess) e = e2;
  if (e != cudaSuccess) return cuda_fail(e, "voxelization", __FILE__, __LINE__);
  if (flags[0]) return fail(PFDTD_ERR_UNSUPPORTED, "more than 64 surface crossings in a column");
  return PFDTD_OK;
}
