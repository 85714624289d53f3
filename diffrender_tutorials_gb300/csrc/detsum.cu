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
constexpr int DS_TR_BLOCKS = 256;                      // blocks of the dense transform sums

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

// ---- segmented sums in a fixed shape ---------------------------------------
// The sorted records are cut into chunks of DS_SEG_CHUNK; a warp owns a
// chunk and each lane a contiguous run of DS_SEG_LANE records.  A lane sums
// its records sequentially: a run of one key that starts and ends inside the
// lane's range is a whole segment (the keys are sorted) and goes straight to
// the gradient; the lane's first and last runs are fragments.  Lane 0 merges
// the 32 lanes' fragments in lane order the same way, leaving the chunk's
// first and last runs as fragments in two slots per chunk.  A second pass
// merges those fragments in order the same way (chunks of 2,048 slots), and
// one warp merges that pass's fragments.  The association order of every
// sum depends only on the record count and the sorted keys.
constexpr int DS_SEG_LANE = 64;
constexpr int DS_SEG_CHUNK = 32 * DS_SEG_LANE;

__device__ __forceinline__ void frag_add(float* grad, uint32_t k, float x, float y, float z) {
  grad[k + 0] += x;
  grad[k + 1] += y;
  grad[k + 2] += z;
}

// Sequential pass over items [b, e) of a sorted sequence given by get(i) ->
// (key, value); keys equal to kNoKey are skipped.  Runs strictly inside the
// range are written to grad; the first and last runs are returned (first ==
// last when the range holds a single run: then last.key = kNoKey).
template <class Get>
__device__ __forceinline__ void seq_runs(Get get, int b, int e, float* grad, DetFrag& first, DetFrag& last) {
  first.key = last.key = kNoKey;
  uint32_t ck = kNoKey;
  float sx = 0.0f, sy = 0.0f, sz = 0.0f;
  bool have_first = false;
  for (int i = b; i < e; i++) {
    uint32_t k;
    float4 v;
    get(i, k, v);
    if (k == kNoKey) continue;
    if (k != ck) {
      if (ck != kNoKey) {
        if (!have_first) {
          first = DetFrag{ck, sx, sy, sz};
          have_first = true;
        } else {
          frag_add(grad, ck, sx, sy, sz);
        }
      }
      ck = k;
      sx = sy = sz = 0.0f;
    }
    sx += v.x;
    sy += v.y;
    sz += v.z;
  }
  if (ck != kNoKey) {
    if (!have_first) first = DetFrag{ck, sx, sy, sz};
    else last = DetFrag{ck, sx, sy, sz};
  }
}

// Lane 0 merges the lanes' (first, last) fragments in lane order.  With
// `whole` the sequence has no neighbours (its first and last runs are whole
// segments); otherwise they are returned as the chunk's fragments.
__device__ __forceinline__ void merge_lane_frags(const DetFrag* f, float* grad, bool whole, DetFrag& cf, DetFrag& cl) {
  cf.key = cl.key = kNoKey;
  uint32_t ck = kNoKey;
  float sx = 0.0f, sy = 0.0f, sz = 0.0f;
  bool have_first = false;
  for (int j = 0; j < 64; j++) {
    const DetFrag g = f[j];
    if (g.key == kNoKey) continue;
    if (g.key != ck) {
      if (ck != kNoKey) {
        if (!have_first && !whole) {
          cf = DetFrag{ck, sx, sy, sz};
          have_first = true;
        } else {
          frag_add(grad, ck, sx, sy, sz);
          have_first = true;
        }
      }
      ck = g.key;
      sx = sy = sz = 0.0f;
    }
    sx += g.x;
    sy += g.y;
    sz += g.z;
  }
  if (ck != kNoKey) {
    if (whole) frag_add(grad, ck, sx, sy, sz);
    else if (!have_first) cf = DetFrag{ck, sx, sy, sz};
    else cl = DetFrag{ck, sx, sy, sz};
  }
}

// FRAGS: the input is the previous level's chunk fragments (two slots per
// chunk of the *n_ptr sorted records) instead of the records.
template <bool FRAGS>
__global__ void __launch_bounds__(DS_THREADS) k_ds_seg_chunks(const uint32_t* key, const int* idx, const int* n_ptr,
                                                              const float4* val, const DetFrag* in, float* grad,
                                                              DetFrag* chunk_frags) {
  __shared__ DetFrag sf[DS_THREADS / 32][64];
  const int n = FRAGS ? 2 * ((*n_ptr + DS_SEG_CHUNK - 1) / DS_SEG_CHUNK) : *n_ptr;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int n_chunks = (n + DS_SEG_CHUNK - 1) / DS_SEG_CHUNK;
  const int warps = gridDim.x * (DS_THREADS / 32);
  for (int c = blockIdx.x * (DS_THREADS / 32) + w; c < n_chunks; c += warps) {
    const int b = min(n, c * DS_SEG_CHUNK + lane * DS_SEG_LANE), e = min(n, b + DS_SEG_LANE);
    DetFrag f0, f1;
    seq_runs([&](int i, uint32_t& k, float4& v) {
      if (FRAGS) {
        const DetFrag g = in[i];
        k = g.key;
        v = make_float4(g.x, g.y, g.z, 0.0f);
      } else {
        k = key[i];
        v = val[idx[i]];
      }
    }, b, e, grad, f0, f1);
    sf[w][2 * lane] = f0;
    sf[w][2 * lane + 1] = f1;
    __syncwarp();
    if (lane == 0) {
      DetFrag cf, cl;
      merge_lane_frags(sf[w], grad, false, cf, cl);
      chunk_frags[2 * c] = cf;
      chunk_frags[2 * c + 1] = cl;
    }
    __syncwarp();
  }
}

// One warp: the second level's fragments in order, lanes over contiguous
// ranges of slots, then lane 0.
__global__ void __launch_bounds__(32) k_ds_seg_final(const int* n_ptr, const DetFrag* chunk_frags, float* grad) {
  __shared__ DetFrag sf[64];
  const int n = *n_ptr;
  const int lane = threadIdx.x;
  const int slots1 = 2 * ((n + DS_SEG_CHUNK - 1) / DS_SEG_CHUNK);
  const int slots = 2 * ((slots1 + DS_SEG_CHUNK - 1) / DS_SEG_CHUNK);
  const int per = (slots + 31) / 32;
  const int b = min(slots, lane * per), e = min(slots, b + per);
  DetFrag f0, f1;
  seq_runs([&](int i, uint32_t& k, float4& v) {
    const DetFrag g = chunk_frags[i];
    k = g.key;
    v = make_float4(g.x, g.y, g.z, 0.0f);
  }, b, e, grad, f0, f1);
  sf[2 * lane] = f0;
  sf[2 * lane + 1] = f1;
  __syncwarp();
  if (lane == 0) {
    DetFrag cf, cl;
    merge_lane_frags(sf, grad, true, cf, cl);
  }
}

// Stable radix sort of (key, value) pairs whose count is on the device, keys
// below 2^bits; the pairs are in keys[0]/vals[0] and end in the buffer whose
// index is returned.
int sort_pairs_device(uint32_t* keys[2], int* vals[2], const int* n_ptr, int bits, uint32_t* hist, cudaStream_t s) {
  const int passes = std::max(1, (bits + 7) / 8);
  int cur = 0;
  for (int p = 0; p < passes; p++) {
    k_ds_hist<<<DS_GRID, DS_THREADS, 0, s>>>(keys[cur], n_ptr, 8 * p, hist);
    launch_rs_scan(hist, 256 * DS_GRID, s);
    k_ds_scatter<<<DS_GRID, DS_THREADS, 0, s>>>(keys[cur], vals[cur], keys[cur ^ 1], vals[cur ^ 1], n_ptr, 8 * p, hist);
    count_launch(2);
    cur ^= 1;
  }
  return cur;
}

int64_t det_regions(const Job& J) { return (int64_t)J.dev.item_count + (int64_t)J.n_views * J.dev.edge_samples; }

// Buffers of the deterministic mode for the current views, work items and
// edge-sample count (grow-only).
// Fragment slots of the first level (two per chunk of records, at the
// record capacity); the second level's follow them.
static int64_t det_frag_l1(const Job& J) {
  const int64_t cap = (int64_t)J.dev.item_count * J.dev.rec_item_cap +
                      (int64_t)J.n_views * J.dev.edge_samples * kEdgeRecords;
  return 2 * ((std::max<int64_t>(1, cap) + DS_SEG_CHUNK - 1) / DS_SEG_CHUNK);
}

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
  J.det_part.reserve(scan_scratch((size_t)std::max<int64_t>(1, (regions + DS_CHUNK - 1) / DS_CHUNK)));
  J.det_hist.reserve(scan_scratch(256 * DS_GRID));
  const int64_t l1 = det_frag_l1(J);
  J.det_frag.reserve(l1 + 2 * ((l1 + DS_SEG_CHUNK - 1) / DS_SEG_CHUNK));
  J.det_n.reserve(1);
  // A single transform block among the differentiable meshes (one mesh, one
  // instance): its 12 values per edge sample are summed densely in a fixed
  // order instead of going through the sort as 4 records per sample.
  int blocks = 0;
  J.det_tr_key = -1;
  for (const DLayout& L : J.dlay) {
    blocks += L.instances;
    if (L.instances == 1) J.det_tr_key = (int)(L.base + L.tr_off);
  }
  if (blocks != 1 || J.dev.edge_samples <= 0) J.det_tr_key = -1;
#ifdef DRGB_NO_DENSE_TR
  J.det_tr_key = -1;
#endif
  if (J.det_tr_key >= 0) {
    J.det_tr.reserve(12 * (size_t)J.n_views * J.dev.edge_samples);
    J.det_tr_part.reserve(12 * (size_t)DS_TR_BLOCKS);
  }
  J.dev.det = 1;
  J.dev.rec_key = J.rec_key.p;
  J.dev.rec_val = J.rec_val.p;
  J.dev.rec_count = J.rec_count.p;
  J.dev.det_tr = J.det_tr_key >= 0 ? J.det_tr.p : nullptr;
  J.dev.det_tr_key = J.det_tr_key;
}

void launch_det_clear(const Job& J, cudaStream_t s) {
  DRGB_CUDA(cudaMemsetAsync(J.rec_count.p, 0, sizeof(int) * std::max<int64_t>(1, det_regions(J)), s));
  if (J.det_tr_key >= 0)
    DRGB_CUDA(cudaMemsetAsync(J.det_tr.p, 0, sizeof(float) * 12 * (size_t)J.n_views * J.dev.edge_samples, s));
}

// Dense transform sums: block b adds samples [b*chunk, (b+1)*chunk) (thread t
// every DS_THREADS-th one from t, then a fixed tree), the last kernel adds
// the block sums in block order into the gradient.
__global__ void __launch_bounds__(DS_THREADS) k_ds_tr_blocks(const float* tr, int64_t n, float* part) {
  __shared__ float red[12][DS_THREADS];
  const int64_t chunk = (n + DS_TR_BLOCKS - 1) / DS_TR_BLOCKS;
  const int64_t b0 = blockIdx.x * chunk, b1 = min(n, b0 + chunk);
  float acc[12];
#pragma unroll
  for (int k = 0; k < 12; k++) acc[k] = 0.0f;
  for (int64_t i = b0 + threadIdx.x; i < b1; i += DS_THREADS) {
    const float4* T = reinterpret_cast<const float4*>(tr + 12 * i);
#pragma unroll
    for (int q = 0; q < 3; q++) {
      const float4 v = T[q];
      acc[4 * q] += v.x; acc[4 * q + 1] += v.y; acc[4 * q + 2] += v.z; acc[4 * q + 3] += v.w;
    }
  }
#pragma unroll
  for (int k = 0; k < 12; k++) red[k][threadIdx.x] = acc[k];
  __syncthreads();
  for (int h = DS_THREADS / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h)
#pragma unroll
      for (int k = 0; k < 12; k++) red[k][threadIdx.x] += red[k][threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x < 12) part[12 * blockIdx.x + threadIdx.x] = red[threadIdx.x][0];
}

__global__ void k_ds_tr_final(const float* part, float* grad, int key) {
  const int k = threadIdx.x;
  if (k >= 12) return;
  float s = 0.0f;
  for (int b = 0; b < DS_TR_BLOCKS; b++) s += part[12 * b + k];
  grad[key + k] += s;
}

void launch_det_reduce(const Job& J, int sm_count, cudaStream_t s) {
  const int64_t regions = det_regions(J);
  if (regions <= 0 || J.grad_alloc <= 0) return;
  const int nb = (int)((regions + DS_CHUNK - 1) / DS_CHUNK);
  k_ds_count_sums<<<nb, DS_THREADS, 0, s>>>(J.rec_count.p, regions, J.det_part.p);
  launch_rs_scan(J.det_part.p, nb, s);
  k_ds_compact<<<nb, DS_THREADS, 0, s>>>(J.rec_count.p, regions, J.det_part.p, nb, J.rec_key.p, J.dev.item_count,
                                         J.dev.rec_item_cap, J.det_key[0].p, J.det_idx[0].p, J.det_n.p);
  count_launch(2);
  int bits = 1;
  while (bits < 32 && ((int64_t)1 << bits) < J.grad_alloc) bits++;
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
  // three levels: chunks of records, chunks of their fragments, one warp
  DetFrag* l2 = J.det_frag.p + det_frag_l1(J);
  k_ds_seg_chunks<false><<<std::max(1, sm_count) * 8, DS_THREADS, 0, s>>>(J.det_key[cur].p, J.det_idx[cur].p,
                                                                           J.det_n.p, J.rec_val.p, nullptr, J.grad.p,
                                                                           J.det_frag.p);
  k_ds_seg_chunks<true><<<std::max(1, sm_count), DS_THREADS, 0, s>>>(nullptr, nullptr, J.det_n.p, nullptr,
                                                                      J.det_frag.p, J.grad.p, l2);
  k_ds_seg_final<<<1, 32, 0, s>>>(J.det_n.p, l2, J.grad.p);
  count_launch(3);
  if (J.det_tr_key >= 0) {
    k_ds_tr_blocks<<<DS_TR_BLOCKS, DS_THREADS, 0, s>>>(J.det_tr.p, (int64_t)J.n_views * J.dev.edge_samples,
                                                      J.det_tr_part.p);
    k_ds_tr_final<<<1, 32, 0, s>>>(J.det_tr_part.p, J.grad.p, J.det_tr_key);
    count_launch(2);
  }
}

}  // namespace drgb
