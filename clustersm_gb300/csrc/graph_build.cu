// graph_build.cu — the data graph's CSR built on the device from an edge list.
//
// The reference builds its CSR on the host while it reads the file, with
// four std::map inserts per edge and neighbour lists in file order
// (readGraphToCPU2, io.cu:60-96).  Here an undirected edge list (any order,
// repeats and both orientations allowed) goes to the device, which
//
//   1. writes both directions of every pair as one 64-bit key
//      (source << 32 | target); self-loops become a sentinel that sorts last;
//   2. sorts the keys with a least-significant-digit radix sort, 8 bits per
//      pass, over the bits the vertex count needs (a stable tile scatter:
//      warps rank equal digits with __match_any_sync);
//   3. keeps the first of every run of equal keys, compacts the targets into
//      the neighbour array and counts degrees;
//   4. scans the degrees into 64-bit offsets.
//
// The result is the same sorted, duplicate-free, loop-free CSR as the host
// paths build (gen.cpp build_simple_csr, the upload's sort of file-order
// lists), then handed to the rest of the resident graph's construction.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <vector>

#include "api_internal.cuh"

namespace smg {
namespace {

constexpr int kThreads = 256;              // 8 warps
constexpr int kItems = 8;                  // keys per thread per tile
constexpr uint32_t kTile = kThreads * kItems;  // 2,048 keys per tile
constexpr int kBins = 256;                 // 8-bit digits
constexpr uint32_t kScanItems = 4;
constexpr uint32_t kScanTile = 1024 * kScanItems;

// Device buffer released with its owner.
template <typename T>
struct DevBuf {
  T *p = nullptr;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
  cudaError_t alloc(size_t n) { return cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)); }
};

// Both directions of pair i; a self-loop or an endpoint outside [0, n)
// becomes the sentinel n << 32 (an endpoint outside [0, n) also sets *bad).
__global__ void k_pair_keys(const uint32_t *__restrict__ pairs, uint64_t np, uint32_t n,
                            uint64_t *__restrict__ keys, int *bad) {
  const uint64_t sentinel = static_cast<uint64_t>(n) << 32;
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < np;
       i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const uint2 e = reinterpret_cast<const uint2 *>(pairs)[i];
    uint64_t k0 = sentinel, k1 = sentinel;
    if (e.x >= n || e.y >= n) {
      atomicExch(bad, 1);
    } else if (e.x != e.y) {
      k0 = (static_cast<uint64_t>(e.x) << 32) | e.y;
      k1 = (static_cast<uint64_t>(e.y) << 32) | e.x;
    }
    reinterpret_cast<ulonglong2 *>(keys)[i] = make_ulonglong2(k0, k1);
  }
}

__device__ __forceinline__ uint32_t digit_of(uint64_t k, int shift) { return static_cast<uint32_t>(k >> shift) & 255u; }

// Per tile: how many of its keys carry each digit, stored digit-major
// (counts[d * tiles + tile]) so that one exclusive scan gives every tile's
// first output position per digit.
__global__ void __launch_bounds__(kThreads) k_radix_count(const uint64_t *__restrict__ keys, uint64_t nk, int shift,
                                                          uint32_t *__restrict__ counts, uint32_t tiles) {
  __shared__ uint32_t h[kBins];
  h[threadIdx.x] = 0;
  __syncthreads();
  const uint64_t base = static_cast<uint64_t>(blockIdx.x) * kTile;
#pragma unroll
  for (int i = 0; i < kItems; ++i) {
    const uint64_t idx = base + i * kThreads + threadIdx.x;
    if (idx < nk) atomicAdd(&h[digit_of(__ldg(keys + idx), shift)], 1u);
  }
  __syncthreads();
  counts[static_cast<uint64_t>(threadIdx.x) * tiles + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter of one tile.  Warp w ranks keys [w*256, (w+1)*256) of the
// tile in 8 rounds of 32 consecutive keys: lanes holding the same digit find
// each other with __match_any_sync and take consecutive slots after the
// warp's running count of that digit.  The warps' counts are then turned into
// per-warp bases behind the tile's scanned global position.
__global__ void __launch_bounds__(kThreads) k_radix_scatter(const uint64_t *__restrict__ in, uint64_t *__restrict__ out,
                                                            uint64_t nk, int shift, const uint32_t *__restrict__ pos,
                                                            uint32_t tiles) {
  __shared__ uint32_t wcnt[kThreads / 32][kBins];
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5, lt = (1u << lane) - 1;
#pragma unroll
  for (int w = 0; w < kThreads / 32; ++w) wcnt[w][threadIdx.x] = 0;
  __syncthreads();
  const uint64_t base = static_cast<uint64_t>(blockIdx.x) * kTile + warp * (32u * kItems);
  uint64_t key[kItems];
  uint32_t slot[kItems];
#pragma unroll
  for (int r = 0; r < kItems; ++r) {
    const uint64_t idx = base + r * 32 + lane;
    const bool valid = idx < nk;
    key[r] = valid ? __ldg(in + idx) : 0ull;
    const uint32_t d = valid ? digit_of(key[r], shift) : kBins;  // invalid lanes form their own group
    const uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
    const uint32_t before = valid ? wcnt[warp][d] : 0u;
    slot[r] = before + __popc(peers & lt);
    __syncwarp();
    if (valid && (peers & lt) == 0) wcnt[warp][d] = before + __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  {
    const uint32_t d = threadIdx.x;
    uint32_t run = pos[static_cast<uint64_t>(d) * tiles + blockIdx.x];
#pragma unroll
    for (int w = 0; w < kThreads / 32; ++w) {
      const uint32_t c = wcnt[w][d];
      wcnt[w][d] = run;
      run += c;
    }
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < kItems; ++r) {
    const uint64_t idx = base + r * 32 + lane;
    if (idx < nk) out[wcnt[warp][digit_of(key[r], shift)] + slot[r]] = key[r];
  }
}

// Exclusive scan, in place, of one tile of kScanTile values per block;
// writes each tile's total to sums (if not null).
template <typename T>
__global__ void __launch_bounds__(1024) k_scan_tiles(T *a, uint64_t n, T *sums) {
  __shared__ T warp_tot[32];
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint64_t base = static_cast<uint64_t>(blockIdx.x) * kScanTile + threadIdx.x * kScanItems;
  T v[kScanItems], own = 0;
#pragma unroll
  for (uint32_t i = 0; i < kScanItems; ++i) {
    v[i] = base + i < n ? a[base + i] : T(0);
    own += v[i];
  }
  T incl = own;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const T t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
    if (lane >= static_cast<uint32_t>(o)) incl += t;
  }
  if (lane == 31) warp_tot[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    T w = warp_tot[lane], wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const T t = __shfl_up_sync(0xFFFFFFFFu, wi, o);
      if (lane >= static_cast<uint32_t>(o)) wi += t;
    }
    warp_tot[lane] = wi - w;  // exclusive prefix of the warps' totals
    if (lane == 31 && sums) sums[blockIdx.x] = wi;
  }
  __syncthreads();
  T run = warp_tot[warp] + incl - own;
#pragma unroll
  for (uint32_t i = 0; i < kScanItems; ++i) {
    if (base + i < n) a[base + i] = run;
    run += v[i];
  }
}

template <typename T>
__global__ void __launch_bounds__(1024) k_scan_add(T *a, uint64_t n, const T *sums) {
  const T add = sums[blockIdx.x];
  const uint64_t base = static_cast<uint64_t>(blockIdx.x) * kScanTile + threadIdx.x * kScanItems;
#pragma unroll
  for (uint32_t i = 0; i < kScanItems; ++i)
    if (base + i < n) a[base + i] += add;
}

// Exclusive scan of a[0, n) in place (any n): tiles, then the tiles' totals
// recursively, then the totals added back.
template <typename T>
cudaError_t scan_exclusive(T *a, uint64_t n, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const uint64_t tiles = (n + kScanTile - 1) / kScanTile;
  if (tiles == 1) {
    k_scan_tiles<T><<<1, 1024, 0, s>>>(a, n, nullptr);
    return cudaGetLastError();
  }
  DevBuf<T> sums;
  cudaError_t e = sums.alloc(tiles);
  if (e != cudaSuccess) return e;
  k_scan_tiles<T><<<static_cast<uint32_t>(tiles), 1024, 0, s>>>(a, n, sums.p);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = scan_exclusive<T>(sums.p, tiles, s)) != cudaSuccess) return e;
  k_scan_add<T><<<static_cast<uint32_t>(tiles), 1024, 0, s>>>(a, n, sums.p);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  return cudaStreamSynchronize(s);  // `sums` is released on return
}

// keep[i] = 1 for the first key of every run of equal keys that is not the
// sentinel (its source is n).
__global__ void k_mark_first(const uint64_t *__restrict__ keys, uint64_t nk, uint32_t n, uint32_t *__restrict__ keep) {
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < nk;
       i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const uint64_t k = keys[i];
    keep[i] = (k >> 32) < n && (i == 0 || keys[i - 1] != k) ? 1u : 0u;
  }
}

// The kept targets go to their scanned positions; degrees are counted with
// one atomic per run of equal sources in a warp (the keys are sorted, so a
// warp's entries mostly share one source).
__global__ void k_compact(const uint64_t *__restrict__ keys, const uint32_t *__restrict__ keep,
                          const uint32_t *__restrict__ at, uint64_t nk, uint32_t *__restrict__ adj,
                          unsigned long long *__restrict__ deg) {
  const uint32_t lane = threadIdx.x & 31, lt = (1u << lane) - 1;
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t i0 = blockIdx.x * static_cast<uint64_t>(blockDim.x); i0 < nk; i0 += stride) {
    const uint64_t i = i0 + threadIdx.x;
    const bool kept = i < nk && keep[i];
    const uint64_t k = kept ? keys[i] : 0ull;
    if (kept) adj[at[i]] = static_cast<uint32_t>(k);
    const uint32_t src = kept ? static_cast<uint32_t>(k >> 32) : 0xFFFFFFFFu;
    const uint32_t peers = __match_any_sync(0xFFFFFFFFu, src);
    if (kept && (peers & lt) == 0) atomicAdd(deg + src, static_cast<unsigned long long>(__popc(peers)));
  }
}

__global__ void k_narrow(const unsigned long long *__restrict__ off64, uint32_t *__restrict__ off32, uint64_t n1) {
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n1;
       i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
    off32[i] = static_cast<uint32_t>(off64[i]);
}

uint32_t bits_for(uint64_t x) {  // bits needed to write values 0..x
  uint32_t b = 0;
  while (b < 64 && (x >> b)) ++b;
  return std::max<uint32_t>(b, 1);
}

}  // namespace

// Sorted, duplicate-free CSR of an undirected edge list, on the device:
// off64 [n+1] (64-bit offsets) and adj [m2].  Used by smg_graph_build.
smg_status build_csr_device(smg_ctx *c, uint32_t n, uint64_t np, const uint32_t *pairs_host,
                            unsigned long long **off64_out, uint32_t **adj_out, uint64_t *m2_out) {
  cudaStream_t s = c->stream;
  const int grid = c->num_sms * 8;
  const uint64_t nk = 2 * np;
  DevBuf<uint32_t> pairs;
  DevBuf<uint64_t> keys, alt;
  DevBuf<int> bad;
  SMG_CUDA(pairs.alloc(2 * np));
  SMG_CUDA(keys.alloc(nk));
  SMG_CUDA(alt.alloc(nk));
  SMG_CUDA(bad.alloc(1));
  SMG_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), s));
  if (np) SMG_CUDA(cudaMemcpyAsync(pairs.p, pairs_host, 2 * np * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
  k_pair_keys<<<grid, 256, 0, s>>>(pairs.p, np, n, keys.p, bad.p);
  SMG_CUDA(cudaGetLastError());
  int hbad = 0;
  SMG_CUDA(cudaMemcpyAsync(&hbad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  SMG_CUDA(cudaStreamSynchronize(s));
  if (hbad) return fail(SMG_ERR_INVALID, "an edge endpoint is not below num_vertices");
  cudaFree(pairs.p);
  pairs.p = nullptr;

  // targets occupy bits [0, 32) (only the low bits(n-1) vary), sources
  // [32, 64) (bits(n) of them: the sentinel's source is n)
  const uint64_t tiles64 = (nk + kTile - 1) / kTile;
  const uint32_t tiles = static_cast<uint32_t>(std::max<uint64_t>(tiles64, 1));
  DevBuf<uint32_t> cnt;
  SMG_CUDA(cnt.alloc(static_cast<uint64_t>(kBins) * tiles));
  std::vector<int> shifts;
  for (uint32_t b = 0; b < bits_for(n ? n - 1 : 0); b += 8) shifts.push_back(static_cast<int>(b));
  for (uint32_t b = 0; b < bits_for(n); b += 8) shifts.push_back(32 + static_cast<int>(b));
  uint64_t *src = keys.p, *dst = alt.p;
  if (nk) {
    for (int sh : shifts) {
      k_radix_count<<<tiles, kThreads, 0, s>>>(src, nk, sh, cnt.p, tiles);
      SMG_CUDA(cudaGetLastError());
      SMG_CUDA(scan_exclusive<uint32_t>(cnt.p, static_cast<uint64_t>(kBins) * tiles, s));
      k_radix_scatter<<<tiles, kThreads, 0, s>>>(src, dst, nk, sh, cnt.p, tiles);
      SMG_CUDA(cudaGetLastError());
      std::swap(src, dst);
    }
  }
  cudaFree(cnt.p);
  cnt.p = nullptr;

  // first of each run, scanned into positions (alt's memory, now free, holds them)
  uint32_t *keep = reinterpret_cast<uint32_t *>(dst);
  uint32_t *at = keep + nk;
  k_mark_first<<<grid, 256, 0, s>>>(src, nk, n, keep);
  SMG_CUDA(cudaGetLastError());
  SMG_CUDA(cudaMemcpyAsync(at, keep, nk * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
  SMG_CUDA(scan_exclusive<uint32_t>(at, nk, s));
  uint32_t last_at = 0, last_keep = 0;
  if (nk) {
    SMG_CUDA(cudaMemcpyAsync(&last_at, at + nk - 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    SMG_CUDA(cudaMemcpyAsync(&last_keep, keep + nk - 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  }
  SMG_CUDA(cudaStreamSynchronize(s));
  const uint64_t m2 = static_cast<uint64_t>(last_at) + last_keep;
  DevBuf<uint32_t> adj;
  DevBuf<unsigned long long> off;
  SMG_CUDA(adj.alloc(m2));
  SMG_CUDA(off.alloc(static_cast<uint64_t>(n) + 1));
  SMG_CUDA(cudaMemsetAsync(off.p, 0, (static_cast<uint64_t>(n) + 1) * sizeof(unsigned long long), s));
  if (nk) {
    k_compact<<<grid, 256, 0, s>>>(src, keep, at, nk, adj.p, off.p);
    SMG_CUDA(cudaGetLastError());
  }
  SMG_CUDA(scan_exclusive<unsigned long long>(off.p, static_cast<uint64_t>(n) + 1, s));
  SMG_CUDA(cudaStreamSynchronize(s));
  *off64_out = off.p;
  *adj_out = adj.p;
  off.p = nullptr;
  adj.p = nullptr;
  *m2_out = m2;
  return SMG_OK;
}

smg_status narrow_offsets(const unsigned long long *off64, uint32_t *off32, uint64_t n1, cudaStream_t s, int num_sms) {
  k_narrow<<<num_sms * 8, 256, 0, s>>>(off64, off32, n1);
  SMG_CUDA(cudaGetLastError());
  return SMG_OK;
}

}  // namespace smg
