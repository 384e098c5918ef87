// Connectivity builder on the GPU: the O(n) part of mcfd_build_faces — keying
// and pairing every (cell, local face) slot — as integer kernels over a
// device hash table.  Boundary grouping, periodic matching and the boundary
// order run on the host over the free slots (O(n^(2/3))) in the host
// builder's code, so both builders give the same faces index for index.
//
//   slot_keys_kernel  one thread per cell: the sorted corner ids of each
//                     local face (hex faces in CGNS order, tet faces in
//                     Tetrahedron4::faces_ order), 4 x 32 bits per slot
//   insert_kernel     one thread per slot: linear probing into a table of
//                     64-bit words packing (hash, first slot); a slot whose
//                     key is already present (checked on the full key) takes
//                     the entry's second word; a third one is an error
//   mark_kernel       holder = the slot of the lower cell id (the shuffler's
//                     [i_cell_small, i_cell_large] adjacency); free slots
//   exclusive scans   face and free-slot positions in (cell, side) order, so
//                     interior faces come out sorted by (holder, side)
//   emit_kernel       the face records
// Every probe loop is bounded by the table size; a run that hits the bound
// or finds a face shared by three cells reports it through an error word.
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "mesh_build_gpu.hpp"

namespace mcfd {
namespace {

// Local faces by family (hexahedron, tetrahedron, wedge, pyramid), the
// tables of geometry.hpp cell_face_corners; -1 ends a triangle.
__constant__ int8_t kFacesD[4][6][4] = {
    {{0, 3, 2, 1}, {0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {0, 4, 7, 3}, {4, 5, 6, 7}},
    {{0, 2, 1, -1}, {0, 1, 3, -1}, {0, 3, 2, -1}, {1, 2, 3, -1}, {-1, -1, -1, -1}, {-1, -1, -1, -1}},
    {{0, 2, 1, -1}, {3, 4, 5, -1}, {0, 1, 4, 3}, {1, 2, 5, 4}, {0, 3, 5, 2}, {-1, -1, -1, -1}},
    {{0, 3, 2, 1}, {0, 1, 4, -1}, {1, 2, 4, -1}, {2, 3, 4, -1}, {3, 0, 4, -1}, {-1, -1, -1, -1}}};
__constant__ int8_t kNFacesD[4] = {6, 4, 5, 5};

constexpr uint64_t kNone = ~0ull;
enum : unsigned { kErrThree = 1u, kErrProbe = 2u, kErrSameCell = 4u };

// family of a cell: 0 hexahedron (Hex8/20/27), 1 tetrahedron (Tet4/10),
// 2 wedge (Wedge6/15/18), 3 pyramid (Pyra5/13/14) (enum mcfd_cell_type)
__device__ __forceinline__ int family(const int32_t *type, int64_t c) {
  if (!type) return 0;
  const int t = type[c];
  return (t == 1 || t == 3) ? 1 : (t == 5 || t == 7 || t == 8) ? 2 : (t == 6 || t == 9 || t == 10) ? 3 : 0;
}

__device__ __forceinline__ void sort4(uint32_t *k) {
#define MCFD_SWAP(a, b) \
  if (k[a] > k[b]) { const uint32_t t_ = k[a]; k[a] = k[b]; k[b] = t_; }
  MCFD_SWAP(0, 1) MCFD_SWAP(2, 3) MCFD_SWAP(0, 2) MCFD_SWAP(1, 3) MCFD_SWAP(1, 2)
#undef MCFD_SWAP
}

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
  x ^= x >> 30; x *= 0xbf58476d1ce4e5b9ull;
  x ^= x >> 27; x *= 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

__device__ __forceinline__ uint64_t key_hash(const uint4 &k) {
  return mix64(mix64(((uint64_t)k.x << 32 | k.y) + 0x9e3779b97f4a7c15ull) ^ ((uint64_t)k.z << 32 | k.w));
}

__device__ __forceinline__ bool same(const uint4 &a, const uint4 &b) {
  return a.x == b.x && a.y == b.y && a.z == b.z && a.w == b.w;
}

__global__ void slot_keys_kernel(const int64_t *cell_nodes, int64_t stride, const int32_t *type,
                                 const int64_t *slot_off, int64_t n_cells, uint4 *keys,
                                 int64_t *slot_cell, int8_t *slot_side) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n_cells) return;
  const int fam = family(type, c);
  const int64_t base = slot_off[c];
  for (int s = 0; s < kNFacesD[fam]; ++s) {
    uint32_t k[4] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu};
    for (int v = 0; v < 4 && kFacesD[fam][s][v] >= 0; ++v)
      k[v] = (uint32_t)cell_nodes[c * stride + kFacesD[fam][s][v]];
    sort4(k);
    keys[base + s] = make_uint4(k[0], k[1], k[2], k[3]);
    slot_cell[base + s] = c;
    slot_side[base + s] = (int8_t)s;
  }
}

__global__ void insert_kernel(const uint4 *keys, int64_t n_slots, unsigned long long *first,
                              unsigned long long *second, uint64_t mask, int64_t *entry,
                              unsigned *err) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_slots) return;
  const uint4 key = keys[i];
  const uint64_t h = key_hash(key);
  const uint32_t tag = (uint32_t)(h >> 32) | 1u;
  const unsigned long long mine = ((unsigned long long)tag << 32) | (uint32_t)i;
  uint64_t pos = h & mask;
  for (uint64_t probe = 0; probe <= mask; ++probe) {
    const unsigned long long old = atomicCAS(&first[pos], 0ull, mine);
    if (old == 0ull) {
      entry[i] = (int64_t)pos;
      return;
    }
    if ((uint32_t)(old >> 32) == tag && same(keys[(uint32_t)old], key)) {
      const unsigned long long prev = atomicCAS(&second[pos], kNone, (unsigned long long)i);
      if (prev != kNone) atomicOr(err, kErrThree);
      entry[i] = (int64_t)pos;
      return;
    }
    pos = (pos + 1) & mask;
  }
  atomicOr(err, kErrProbe);
  entry[i] = -1;
}

__global__ void mark_kernel(const unsigned long long *first, const unsigned long long *second,
                            const int64_t *entry, const int64_t *slot_cell, int64_t n_slots,
                            int32_t *holder, int32_t *lone, int64_t *partner, unsigned *err) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_slots) return;
  holder[i] = 0;
  lone[i] = 0;
  const int64_t pos = entry[i];
  if (pos < 0) return;
  const int64_t a = (int64_t)(uint32_t)first[pos];
  const unsigned long long b = second[pos];
  if (b == kNone) {
    lone[i] = 1;
    return;
  }
  const int64_t other = i == a ? (int64_t)b : a;
  const int64_t ci = slot_cell[i], co = slot_cell[other];
  if (ci == co) atomicOr(err, kErrSameCell);
  holder[i] = ci < co ? 1 : 0;
  partner[i] = other;
}

__global__ void emit_kernel(const int32_t *holder, const int32_t *lone, const int64_t *hpos,
                            const int64_t *lpos, const int64_t *partner, const int64_t *slot_cell,
                            const int8_t *slot_side, int64_t n_slots, int64_t *inner_cells,
                            int32_t *inner_sides, int64_t *lone_cells, int32_t *lone_sides) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_slots) return;
  if (holder[i]) {
    const int64_t f = hpos[i], o = partner[i];
    inner_cells[2 * f] = slot_cell[i];
    inner_cells[2 * f + 1] = slot_cell[o];
    inner_sides[2 * f] = slot_side[i];
    inner_sides[2 * f + 1] = slot_side[o];
  } else if (lone[i]) {
    const int64_t l = lpos[i];
    lone_cells[l] = slot_cell[i];
    lone_sides[l] = slot_side[i];
  }
}

// Exclusive prefix sums of int32 marks into int64 positions: per-block scans
// of 1024 values, a recursive scan of the block totals, then the offsets.
constexpr int kScanThreads = 256, kScanItems = 4, kScanBlock = kScanThreads * kScanItems;

template <class T>
__global__ void block_scan_kernel(const T *in, int64_t *out, int64_t *block_sums, int64_t n) {
  __shared__ int64_t s_warp[kScanThreads / 32];
  const int64_t base = (int64_t)blockIdx.x * kScanBlock + threadIdx.x * kScanItems;
  int64_t v[kScanItems], sum = 0;
  for (int j = 0; j < kScanItems; ++j) {
    v[j] = base + j < n ? (int64_t)in[base + j] : 0;
    sum += v[j];
  }
  // inclusive scan of the per-thread sums within the block
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int64_t x = sum;
  for (int d = 1; d < 32; d <<= 1) {
    const int64_t y = __shfl_up_sync(0xffffffffu, x, d);
    if (lane >= d) x += y;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int64_t w = lane < kScanThreads / 32 ? s_warp[lane] : 0;
    for (int d = 1; d < 32; d <<= 1) {
      const int64_t y = __shfl_up_sync(0xffffffffu, w, d);
      if (lane >= d) w += y;
    }
    if (lane < kScanThreads / 32) s_warp[lane] = w;
  }
  __syncthreads();
  int64_t run = x - sum + (warp > 0 ? s_warp[warp - 1] : 0);
  for (int j = 0; j < kScanItems; ++j) {
    if (base + j < n) out[base + j] = run;
    run += v[j];
  }
  if (threadIdx.x == kScanThreads - 1) block_sums[blockIdx.x] = run;
}

__global__ void add_offsets_kernel(int64_t *out, const int64_t *offsets, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += offsets[i / kScanBlock];
}

template <class T>
cudaError_t exclusive_scan(const T *in, int64_t *out, int64_t n) {
  if (n <= 0) return cudaSuccess;
  const int64_t nb = (n + kScanBlock - 1) / kScanBlock;
  int64_t *sums = nullptr, *offs = nullptr;
  cudaError_t e = cudaMalloc(&sums, sizeof(int64_t) * nb);
  if (e == cudaSuccess) e = cudaMalloc(&offs, sizeof(int64_t) * nb);
  if (e == cudaSuccess) {
    block_scan_kernel<T><<<(unsigned)nb, kScanThreads>>>(in, out, sums, n);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && nb > 1) {
    e = exclusive_scan<int64_t>(sums, offs, nb);
    if (e == cudaSuccess) {
      add_offsets_kernel<<<(unsigned)((n + 255) / 256), 256>>>(out, offs, n);
      e = cudaGetLastError();
    }
  }
  cudaFree(sums);
  cudaFree(offs);
  return e;
}

}  // namespace

int gpu_pair_slots(int device, const int64_t *cell_nodes, int64_t stride, const int32_t *cell_type,
                   int64_t n_cells, const std::vector<int64_t> &slot_off, GpuPairs *out,
                   std::string *err) {
  const int64_t ns = slot_off.back();
  uint64_t cap = 1;
  while (cap < (uint64_t)(2 * ns)) cap <<= 1;
  if (cudaSetDevice(device) != cudaSuccess) { *err = "cudaSetDevice failed"; return 1; }
  std::vector<void *> allocs;
  cudaError_t e = cudaSuccess;
  auto alloc = [&](void **p, size_t bytes) {
    if (e == cudaSuccess) e = cudaMalloc(p, bytes > 0 ? bytes : 1);
    if (e == cudaSuccess) allocs.push_back(*p);
  };
  int64_t *d_nodes, *d_off, *d_cell, *d_entry, *d_partner, *d_hpos, *d_lpos, *d_icells, *d_lcells;
  int32_t *d_type = nullptr, *d_holder, *d_lone, *d_isides, *d_lsides;
  int8_t *d_side;
  uint4 *d_keys;
  unsigned long long *d_first, *d_second;
  unsigned *d_err;
  alloc((void **)&d_nodes, sizeof(int64_t) * n_cells * stride);
  if (cell_type) alloc((void **)&d_type, sizeof(int32_t) * n_cells);
  alloc((void **)&d_off, sizeof(int64_t) * (n_cells + 1));
  alloc((void **)&d_keys, sizeof(uint4) * ns);
  alloc((void **)&d_cell, sizeof(int64_t) * ns);
  alloc((void **)&d_side, sizeof(int8_t) * ns);
  alloc((void **)&d_entry, sizeof(int64_t) * ns);
  alloc((void **)&d_partner, sizeof(int64_t) * ns);
  alloc((void **)&d_holder, sizeof(int32_t) * ns);
  alloc((void **)&d_lone, sizeof(int32_t) * ns);
  alloc((void **)&d_hpos, sizeof(int64_t) * ns);
  alloc((void **)&d_lpos, sizeof(int64_t) * ns);
  alloc((void **)&d_first, sizeof(unsigned long long) * cap);
  alloc((void **)&d_second, sizeof(unsigned long long) * cap);
  alloc((void **)&d_err, sizeof(unsigned));
  auto done = [&](int rc) {
    for (void *p : allocs) cudaFree(p);
    return rc;
  };
  if (e == cudaSuccess) e = cudaMemcpy(d_nodes, cell_nodes, sizeof(int64_t) * n_cells * stride, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && cell_type) e = cudaMemcpy(d_type, cell_type, sizeof(int32_t) * n_cells, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d_off, slot_off.data(), sizeof(int64_t) * (n_cells + 1), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(d_first, 0, sizeof(unsigned long long) * cap);
  if (e == cudaSuccess) e = cudaMemset(d_second, 0xff, sizeof(unsigned long long) * cap);
  if (e == cudaSuccess) e = cudaMemset(d_err, 0, sizeof(unsigned));
  const unsigned bc = (unsigned)((n_cells + 255) / 256), bs = (unsigned)((ns + 255) / 256);
  if (e == cudaSuccess) {
    slot_keys_kernel<<<bc, 256>>>(d_nodes, stride, d_type, d_off, n_cells, d_keys, d_cell, d_side);
    insert_kernel<<<bs, 256>>>(d_keys, ns, d_first, d_second, cap - 1, d_entry, d_err);
    mark_kernel<<<bs, 256>>>(d_first, d_second, d_entry, d_cell, ns, d_holder, d_lone, d_partner, d_err);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = exclusive_scan<int32_t>(d_holder, d_hpos, ns);
  if (e == cudaSuccess) e = exclusive_scan<int32_t>(d_lone, d_lpos, ns);
  unsigned h_err = 0;
  int64_t last[2] = {0, 0};
  int32_t last_mark[2] = {0, 0};
  if (e == cudaSuccess) e = cudaMemcpy(&h_err, d_err, sizeof(unsigned), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(&last[0], d_hpos + ns - 1, sizeof(int64_t), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(&last[1], d_lpos + ns - 1, sizeof(int64_t), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(&last_mark[0], d_holder + ns - 1, sizeof(int32_t), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(&last_mark[1], d_lone + ns - 1, sizeof(int32_t), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) {
    *err = std::string("GPU face builder: ") + cudaGetErrorString(e);
    return done(1);
  }
  if (h_err & kErrThree) { *err = "a face is shared by more than two cells"; return done(2); }
  if (h_err & kErrSameCell) { *err = "a cell repeats a face"; return done(2); }
  if (h_err & kErrProbe) { *err = "GPU face builder: hash table probe limit reached"; return done(1); }
  const int64_t n_inner = last[0] + last_mark[0], n_lone = last[1] + last_mark[1];
  alloc((void **)&d_icells, sizeof(int64_t) * 2 * n_inner);
  alloc((void **)&d_isides, sizeof(int32_t) * 2 * n_inner);
  alloc((void **)&d_lcells, sizeof(int64_t) * n_lone);
  alloc((void **)&d_lsides, sizeof(int32_t) * n_lone);
  if (e == cudaSuccess) {
    emit_kernel<<<bs, 256>>>(d_holder, d_lone, d_hpos, d_lpos, d_partner, d_cell, d_side, ns, d_icells,
                             d_isides, d_lcells, d_lsides);
    e = cudaGetLastError();
  }
  out->inner_cells.resize(2 * n_inner);
  out->inner_sides.resize(2 * n_inner);
  out->lone_cells.resize(n_lone);
  out->lone_sides.resize(n_lone);
  if (e == cudaSuccess && n_inner)
    e = cudaMemcpy(out->inner_cells.data(), d_icells, sizeof(int64_t) * 2 * n_inner, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && n_inner)
    e = cudaMemcpy(out->inner_sides.data(), d_isides, sizeof(int32_t) * 2 * n_inner, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && n_lone)
    e = cudaMemcpy(out->lone_cells.data(), d_lcells, sizeof(int64_t) * n_lone, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && n_lone)
    e = cudaMemcpy(out->lone_sides.data(), d_lsides, sizeof(int32_t) * n_lone, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) {
    *err = std::string("GPU face builder: ") + cudaGetErrorString(e);
    return done(1);
  }
  return done(0);
}

}  // namespace mcfd
