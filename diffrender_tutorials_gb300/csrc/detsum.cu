// Deterministic gradient reduction: a vertex-sorted segmented reduction of
// the gradient records written by the pixel and edge kernels in
// deterministic mode.
//
//   1. count scan   exclusive scan of the per-region record counts (work
//                   items in item order, then edge samples in (view, sample)
//                   order) -- integers, so the offsets are exact;
//   2. compaction   each region's records go to dense (key, slot) pairs at
//                   its offset, in the order the producer wrote them;
//   3. sort         stable LSD radix sort of the pairs by gradient index
//                   (8-bit digits, a fixed grid whose blocks own contiguous
//                   chunks, so ties keep their dense order);
//   4. segments     the first record of each gradient index sums its segment
//                   in sorted order and adds the 3 floats to the gradient.
//
// Every step is independent of scheduling: the same inputs give the same
// gradient bits on every run, alone or in a batch.  The reference sums its
// per-thread gradient copies sequentially (src/drender.h:380-424); the order
// here is another fixed order.
#include "engine.h"

namespace drgb {

void launch_rs_scan(uint32_t* hist, int m, cudaStream_t s);

constexpr int DS_THREADS = 256;
constexpr int DS_PER_THREAD = 8;
constexpr int DS_CHUNK = DS_THREADS * DS_PER_THREAD;  // regions per block of the count scan
constexpr int DS_GRID = 512;                           // blocks of the radix sort

__device__ __forceinline__ int64_t region_slot(int64_t r, int item_count, int item_cap) {
  return r < item_count ? r * item_cap
                        : (int64_t)item_count * item_cap + (r - item_count) * (int64_t)kEdgeRecords;
}

__global__ void __launch_bounds__(DS_THREADS) k_ds_count_sums(const int* count, int64_t n_regions, uint32_t* part) {
  __shared__ uint32_t red[DS_THREADS];
  const int64_t base = (int64_t)blockIdx.x * DS_CHUNK;
  uint32_t s = 0;
  for (int i = threadIdx.x; i < DS_CHUNK; i += DS_THREADS) {
    const int64_t r = base + i;
    if (r < n_regions) s += (uint32_t)count[r];
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = DS_THREADS / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// part holds the exclusive block offsets.  Thread t of block b owns regions
// [b*CHUNK + 8t, +8).
__global__ void __launch_bounds__(DS_THREADS) k_ds_compact(const int* count, int64_t n_regions, const uint32_t* part,
                                                           int n_blocks, const uint32_t* rec_key, int item_count,
                                                           int item_cap, uint32_t* dkey, int* didx, int* n_out) {
  __shared__ uint32_t sc[DS_THREADS];
  const int64_t base = (int64_t)blockIdx.x * DS_CHUNK + (int64_t)threadIdx.x * DS_PER_THREAD;
  int c[DS_PER_THREAD];
  uint32_t tsum = 0;
#pragma unroll
  for (int k = 0; k < DS_PER_THREAD; k++) {
    const int64_t r = base + k;
    c[k] = r < n_regions ? count[r] : 0;
    tsum += (uint32_t)c[k];
  }
  sc[threadIdx.x] = tsum;
  __syncthreads();
  for (int o = 1; o < DS_THREADS; o <<= 1) {
    const uint32_t v = threadIdx.x >= o ? sc[threadIdx.x - o] : 0u;
    __syncthreads();
    sc[threadIdx.x] += v;
    __syncthreads();
  }
  uint32_t off = part[blockIdx.x] + sc[threadIdx.x] - tsum;
#pragma unroll
  for (int k = 0; k < DS_PER_THREAD; k++) {
    const int64_t slot = region_slot(base + k, item_count, item_cap);
    for (int j = 0; j < c[k]; j++, off++) {
      dkey[off] = rec_key[slot + j];
      didx[off] = (int)(slot + j);
    }
  }
  if (blockIdx.x == n_blocks - 1 && threadIdx.x == DS_THREADS - 1) *n_out = (int)off;
}

__device__ __forceinline__ void ds_chunk(int n, int& b0, int& b1) {
  const int chunk = (n + DS_GRID - 1) / DS_GRID;
  b0 = min(n, (int)blockIdx.x * chunk);
  b1 = min(n, b0 + chunk);
}

__global__ void __launch_bounds__(DS_THREADS) k_ds_hist(const uint32_t* keys, const int* n_ptr, int shift,
                                                        uint32_t* hist) {
  __shared__ uint32_t h[256];
  int b0, b1;
  ds_chunk(*n_ptr, b0, b1);
  h[threadIdx.x] = 0;
  __syncthreads();
  for (int i = b0 + threadIdx.x; i < b1; i += DS_THREADS) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
  __syncthreads();
  hist[threadIdx.x * DS_GRID + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter of one block's chunk, 256 keys at a time: rank within the
// warp from __match_any_sync, then the counts of the lower warps.
__global__ void __launch_bounds__(DS_THREADS) k_ds_scatter(const uint32_t* kin, const int* vin, uint32_t* kout,
                                                           int* vout, const int* n_ptr, int shift,
                                                           const uint32_t* hist) {
  __shared__ uint32_t offs[256];
  __shared__ uint32_t wcnt[DS_THREADS / 32][257];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  int b0, b1;
  ds_chunk(*n_ptr, b0, b1);
  offs[tid] = hist[tid * DS_GRID + blockIdx.x];
  const unsigned lt = (1u << lane) - 1u;
  for (int t0 = b0; t0 < b1; t0 += DS_THREADS) {
    for (int i = tid; i < (DS_THREADS / 32) * 257; i += DS_THREADS) (&wcnt[0][0])[i] = 0u;
    __syncthreads();
    const int idx = t0 + tid;
    const bool valid = idx < b1;
    const uint32_t key = valid ? kin[idx] : 0u;
    const int val = valid ? vin[idx] : 0;
    const uint32_t digit = valid ? ((key >> shift) & 255u) : 256u;
    const unsigned peers = __match_any_sync(0xffffffffu, digit);
    const uint32_t rank = __popc(peers & lt);
    if ((__ffs(peers) - 1) == lane) wcnt[warp][digit] = __popc(peers);
    __syncthreads();
    if (valid) {
      uint32_t off = offs[digit] + rank;
      for (int w = 0; w < warp; w++) off += wcnt[w][digit];
      kout[off] = key;
      vout[off] = val;
    }
    __syncthreads();
    uint32_t tot = 0;
    for (int w = 0; w < DS_THREADS / 32; w++) tot += wcnt[w][tid];
    offs[tid] += tot;
    __syncthreads();
  }
}

__global__ void __launch_bounds__(DS_THREADS) k_ds_segments(const uint32_t* key, const int* idx, const int* n_ptr,
                                                            const float4* val, float* grad) {
  const int n = *n_ptr;
  const int stride = gridDim.x * blockDim.x;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const uint32_t k = key[i];
    if (i > 0 && key[i - 1] == k) continue;
    float sx = 0.0f, sy = 0.0f, sz = 0.0f;
    for (int j = i; j < n && key[j] == k; j++) {
      const float4 v = val[idx[j]];
      sx += v.x;
      sy += v.y;
      sz += v.z;
    }
    grad[k + 0] += sx;
    grad[k + 1] += sy;
    grad[k + 2] += sz;
  }
}

int64_t det_regions(const Job& J) { return (int64_t)J.dev.item_count + (int64_t)J.n_views * J.dev.edge_samples; }

// Buffers of the deterministic mode for the current views, work items and
// edge-sample count (grow-only).
void det_buffers(Job& J, cudaStream_t s) {
  (void)s;
  const int NS = J.tile_w * J.tile_h * J.S;
  J.dev.rec_item_cap = item_record_cap(J.mode, NS);
  const int64_t regions = det_regions(J);
  const int64_t cap = (int64_t)J.dev.item_count * J.dev.rec_item_cap +
                      (int64_t)J.n_views * J.dev.edge_samples * kEdgeRecords;
  if (cap >= (int64_t)INT32_MAX) throw CudaError("deterministic mode: too many gradient records for one call", DRGB_ERR_UNSUPPORTED);
  J.rec_key.reserve(std::max<int64_t>(1, cap));
  J.rec_val.reserve(std::max<int64_t>(1, cap));
  J.rec_count.reserve(std::max<int64_t>(1, regions));
  for (int b = 0; b < 2; b++) {
    J.det_key[b].reserve(std::max<int64_t>(1, cap));
    J.det_idx[b].reserve(std::max<int64_t>(1, cap));
  }
  J.det_part.reserve(std::max<int64_t>(1, (regions + DS_CHUNK - 1) / DS_CHUNK));
  J.det_hist.reserve(256 * DS_GRID);
  J.det_n.reserve(1);
  J.dev.det = 1;
  J.dev.rec_key = J.rec_key.p;
  J.dev.rec_val = J.rec_val.p;
  J.dev.rec_count = J.rec_count.p;
}

void launch_det_clear(const Job& J, cudaStream_t s) {
  DRGB_CUDA(cudaMemsetAsync(J.rec_count.p, 0, sizeof(int) * std::max<int64_t>(1, det_regions(J)), s));
}

void launch_det_reduce(const Job& J, int sm_count, cudaStream_t s) {
  const int64_t regions = det_regions(J);
  if (regions <= 0 || J.grad_total <= 0) return;
  const int nb = (int)((regions + DS_CHUNK - 1) / DS_CHUNK);
  k_ds_count_sums<<<nb, DS_THREADS, 0, s>>>(J.rec_count.p, regions, J.det_part.p);
  launch_rs_scan(J.det_part.p, nb, s);
  k_ds_compact<<<nb, DS_THREADS, 0, s>>>(J.rec_count.p, regions, J.det_part.p, nb, J.rec_key.p, J.dev.item_count,
                                         J.dev.rec_item_cap, J.det_key[0].p, J.det_idx[0].p, J.det_n.p);
  count_launch(2);
  int bits = 1;
  while (bits < 32 && ((int64_t)1 << bits) < J.grad_total) bits++;
  const int passes = (bits + 7) / 8;
  int cur = 0;
  for (int p = 0; p < passes; p++) {
    k_ds_hist<<<DS_GRID, DS_THREADS, 0, s>>>(J.det_key[cur].p, J.det_n.p, 8 * p, J.det_hist.p);
    launch_rs_scan(J.det_hist.p, 256 * DS_GRID, s);
    k_ds_scatter<<<DS_GRID, DS_THREADS, 0, s>>>(J.det_key[cur].p, J.det_idx[cur].p, J.det_key[cur ^ 1].p,
                                                J.det_idx[cur ^ 1].p, J.det_n.p, 8 * p, J.det_hist.p);
    count_launch(2);
    cur ^= 1;
  }
  k_ds_segments<<<std::max(1, sm_count) * 8, DS_THREADS, 0, s>>>(J.det_key[cur].p, J.det_idx[cur].p, J.det_n.p, J.rec_val.p,
                                               J.grad.p);
  count_launch();
}

}  // namespace drgb
