// Device graph builder: CSR / CSC from an edge list on the GPU.
//
// The reference builds both adjacencies on the host (util.h:44-121,
// edgeListToCSR/CSC; gpugas.h:212-322 copies them up).  Here the edge list
// is copied to the device once and each adjacency is a stable LSD radix
// sort of (key, edge index) pairs, 8-bit digits:
//
//   per pass:  block histograms of the digit (4096 edges per block)
//              -> exclusive scan in digit-major order (a digit's blocks in
//                 order after every smaller digit)
//              -> scatter: each block ranks its edges per digit in edge
//                 order (warp match + per-warp counts), so equal keys keep
//                 edge-list order
//
// which gives the same order as build_adjacency's stable counting sort
// (in-edges of a vertex in edge-list order).  Offsets come from per-key
// counts and an exclusive scan; adjacency and edge data are gathered by the
// sorted edge indices (the permutation).
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "gas_gb300/detail/primitives.cuh"
#include "gas_internal.h"

using gas::internal::cuda_fail;
using gas::internal::fail;

namespace {

constexpr int kBins = 256;
constexpr int kRThreads = 256;
constexpr int kRItems = 16;
constexpr int kRTile = kRThreads * kRItems;  // edges per sort block
constexpr int kSThreads = 1024;
constexpr int kSItems = 8;
constexpr int kSTile = kSThreads * kSItems;  // elements per scan block

__global__ void radix_hist_kernel(const uint32_t *keys, long long n, int shift, int nBlocks,
                                  uint32_t *hist) {
  __shared__ uint32_t h[kBins];
  h[threadIdx.x] = 0u;
  __syncthreads();
  const long long base = (long long)blockIdx.x * kRTile;
#pragma unroll 4
  for (int i = 0; i < kRItems; ++i) {
    const long long idx = base + (long long)i * kRThreads + threadIdx.x;
    if (idx < n) atomicAdd(&h[(keys[idx] >> shift) & (kBins - 1)], 1u);
  }
  __syncthreads();
  hist[(size_t)threadIdx.x * nBlocks + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter of one pass.  vals == null stands for the identity
// (edge index), the first pass's payload.
__global__ void radix_scatter_kernel(const uint32_t *keysIn, const uint32_t *valsIn,
                                     uint32_t *keysOut, uint32_t *valsOut, long long n, int shift,
                                     int nBlocks, const uint32_t *histScan) {
  __shared__ uint32_t run[kBins];
  __shared__ uint32_t warpOff[kRThreads / 32][kBins];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const unsigned ltMask = (1u << lane) - 1u;
  run[tid] = histScan[(size_t)tid * nBlocks + blockIdx.x];
  const long long base = (long long)blockIdx.x * kRTile;
  for (int i = 0; i < kRItems; ++i) {
    const long long idx = base + (long long)i * kRThreads + tid;
    const bool valid = idx < n;
    const uint32_t key = valid ? keysIn[idx] : 0u;
    const uint32_t d = (key >> shift) & (kBins - 1);
    const unsigned peers = __match_any_sync(gas::detail::kFullMask, valid ? d : 0xffffffffu);
    const int rank = __popc(peers & ltMask);
#pragma unroll
    for (int w = 0; w < kRThreads / 32; ++w) warpOff[w][tid] = 0u;
    __syncthreads();
    if (valid && rank == 0) warpOff[warp][d] = (uint32_t)__popc(peers);
    __syncthreads();
    {  // per digit: offsets of the warps of this step, after the earlier steps
      uint32_t r = run[tid];
#pragma unroll
      for (int w = 0; w < kRThreads / 32; ++w) {
        const uint32_t c = warpOff[w][tid];
        warpOff[w][tid] = r;
        r += c;
      }
      run[tid] = r;
    }
    __syncthreads();
    if (valid) {
      const uint32_t pos = warpOff[warp][d] + (uint32_t)rank;
      keysOut[pos] = key;
      valsOut[pos] = valsIn ? valsIn[idx] : (uint32_t)idx;
    }
    __syncthreads();
  }
}

// Block-wide exclusive scan of kSTile elements (in place); the block's
// total goes to sums[blockIdx.x] when sums is non-null.
__global__ void scan_block_kernel(uint32_t *data, long long n, uint32_t *sums) {
  __shared__ uint32_t warpTot[kSThreads / 32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const long long base = (long long)blockIdx.x * kSTile + (long long)tid * kSItems;
  uint32_t v[kSItems];
  uint32_t t = 0u;
#pragma unroll
  for (int k = 0; k < kSItems; ++k) {
    v[k] = base + k < n ? data[base + k] : 0u;
    t += v[k];
  }
  uint32_t incl = t;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(gas::detail::kFullMask, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) warpTot[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = warpTot[lane];
    uint32_t wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(gas::detail::kFullMask, wi, o);
      if (lane >= o) wi += y;
    }
    warpTot[lane] = wi - w;  // exclusive
    if (lane == 31 && sums) sums[blockIdx.x] = wi;
  }
  __syncthreads();
  uint32_t run = warpTot[warp] + incl - t;
#pragma unroll
  for (int k = 0; k < kSItems; ++k) {
    if (base + k < n) data[base + k] = run;
    run += v[k];
  }
}

__global__ void scan_add_kernel(uint32_t *data, long long n, const uint32_t *offs) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) data[i] += offs[i / kSTile];
}

gas_status exclusive_scan(uint32_t *data, long long n, cudaStream_t s) {
  if (n <= 0) return GAS_OK;
  const long long blocks = (n + kSTile - 1) / kSTile;
  if (blocks == 1) {
    scan_block_kernel<<<1, kSThreads, 0, s>>>(data, n, nullptr);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GAS_OK : cuda_fail(e, "graph build scan");
  }
  uint32_t *sums = nullptr;
  cudaError_t e = cudaMallocAsync(&sums, sizeof(uint32_t) * blocks, s);
  if (e != cudaSuccess) return cuda_fail(e, "graph build scan");
  scan_block_kernel<<<(unsigned)blocks, kSThreads, 0, s>>>(data, n, sums);
  gas_status st = exclusive_scan(sums, blocks, s);
  if (st == GAS_OK) {
    scan_add_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(data, n, sums);
    e = cudaGetLastError();
    if (e != cudaSuccess) st = cuda_fail(e, "graph build scan");
  }
  cudaFreeAsync(sums, s);
  return st;
}

__global__ void count_keys_kernel(const int32_t *keys, long long n, uint32_t *cnt) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    atomicAdd(cnt + keys[i], 1u);
}

__global__ void gather_kernel(const int32_t *src, const uint32_t *perm, long long n, int32_t *dst) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    dst[i] = src[perm[i]];
}

// out[p] = in[perm[p]] for elements of `bytes` bytes (word copies when the
// size is a multiple of 4).
__global__ void gather_bytes_kernel(const unsigned char *in, const uint32_t *perm, long long n,
                                    int bytes, unsigned char *out) {
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    const size_t s = (size_t)perm[p] * bytes, d = (size_t)p * bytes;
    if ((bytes & 3) == 0) {
      for (int k = 0; k < bytes; k += 4)
        *reinterpret_cast<uint32_t *>(out + d + k) = *reinterpret_cast<const uint32_t *>(in + s + k);
    } else {
      for (int k = 0; k < bytes; ++k) out[d + k] = in[s + k];
    }
  }
}

// out[perm[p]] = in[p]: back to edge-list order.
__global__ void scatter_bytes_kernel(const unsigned char *in, const uint32_t *perm, long long n,
                                     int bytes, unsigned char *out) {
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    const size_t d = (size_t)perm[p] * bytes, s = (size_t)p * bytes;
    for (int k = 0; k < bytes; ++k) out[d + k] = in[s + k];
  }
}

__global__ void check_ids_kernel(const int32_t *a, const int32_t *b, long long n, int32_t nV,
                                 unsigned long long *firstBad) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    if ((unsigned)a[i] >= (unsigned)nV || (unsigned)b[i] >= (unsigned)nV)
      atomicMin(firstBad, (unsigned long long)i);
}

__global__ void invert_kernel(const uint32_t *perm, long long n, uint32_t *inv) {
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x)
    inv[perm[p]] = (uint32_t)p;
}

__global__ void compose_kernel(const uint32_t *inv, const uint32_t *perm, long long n, int32_t *out) {
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x)
    out[q] = (int32_t)inv[perm[q]];
}

int grid_for(long long n) { return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 152 * 16)); }

}  // namespace

namespace gas {
namespace internal {

gas_status device_first_bad_edge(cudaStream_t s, int32_t nV, int32_t nE, const int32_t *dSrcs,
                                 const int32_t *dDsts, long long *firstBad) {
  *firstBad = -1;
  if (nE <= 0) return GAS_OK;
  unsigned long long *d = nullptr, h = ~0ull;
  cudaError_t e = cudaMallocAsync(&d, sizeof(h), s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d, &h, sizeof(h), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    check_ids_kernel<<<grid_for(nE), 256, 0, s>>>(dSrcs, dDsts, nE, nV, d);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (d) cudaFreeAsync(d, s);
  if (e != cudaSuccess) return cuda_fail(e, "edge id check");
  if (h != ~0ull) *firstBad = (long long)h;
  return GAS_OK;
}

gas_status device_build_adjacency(cudaStream_t s, int32_t nV, int32_t nE, const int32_t *dKey,
                                  const int32_t *dOther, int32_t *dOff, int32_t *dAdj,
                                  uint32_t *dPermOut) {
  cudaError_t e = cudaSuccess;
  const long long n = nE;
  // offsets: per-key counts, exclusive scan over V + 1 entries
  e = cudaMemsetAsync(dOff, 0, sizeof(int32_t) * ((size_t)nV + 1), s);
  if (e != cudaSuccess) return cuda_fail(e, "graph build");
  if (n > 0) count_keys_kernel<<<grid_for(n), 256, 0, s>>>(dKey, n, reinterpret_cast<uint32_t *>(dOff));
  gas_status st = exclusive_scan(reinterpret_cast<uint32_t *>(dOff), (long long)nV + 1, s);
  if (st || n == 0) return st;
  // stable radix sort of (key, edge index)
  int bits = 1;
  while (bits < 31 && (1ll << bits) < nV) ++bits;
  const int passes = (bits + 7) / 8;
  const int nBlocks = (int)((n + kRTile - 1) / kRTile);
  uint32_t *k0 = nullptr, *k1 = nullptr, *v0 = nullptr, *v1 = nullptr, *hist = nullptr;
  e = cudaMallocAsync(&k0, sizeof(uint32_t) * n, s);
  if (e == cudaSuccess) e = cudaMallocAsync(&k1, sizeof(uint32_t) * n, s);
  if (e == cudaSuccess) e = cudaMallocAsync(&v0, sizeof(uint32_t) * n, s);
  if (e == cudaSuccess) e = cudaMallocAsync(&v1, sizeof(uint32_t) * n, s);
  if (e == cudaSuccess) e = cudaMallocAsync(&hist, sizeof(uint32_t) * (size_t)kBins * nBlocks, s);
  const uint32_t *kin = reinterpret_cast<const uint32_t *>(dKey);
  const uint32_t *vin = nullptr;
  uint32_t *kout = k0, *vout = v0;
  for (int p = 0; p < passes && e == cudaSuccess; ++p) {
    radix_hist_kernel<<<nBlocks, kRThreads, 0, s>>>(kin, n, 8 * p, nBlocks, hist);
    e = cudaGetLastError();
    if (e != cudaSuccess) break;
    st = exclusive_scan(hist, (long long)kBins * nBlocks, s);
    if (st) break;
    radix_scatter_kernel<<<nBlocks, kRThreads, 0, s>>>(kin, vin, kout, vout, n, 8 * p, nBlocks,
                                                       hist);
    e = cudaGetLastError();
    kin = kout;
    vin = vout;
    kout = kout == k0 ? k1 : k0;
    vout = vout == v0 ? v1 : v0;
  }
  if (e == cudaSuccess && st == GAS_OK) {
    gather_kernel<<<grid_for(n), 256, 0, s>>>(dOther, vin, n, dAdj);
    e = cudaGetLastError();
    if (e == cudaSuccess && dPermOut)
      e = cudaMemcpyAsync(dPermOut, vin, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, s);
  }
  cudaFreeAsync(k0, s);
  cudaFreeAsync(k1, s);
  cudaFreeAsync(v0, s);
  cudaFreeAsync(v1, s);
  cudaFreeAsync(hist, s);
  if (st) return st;
  return e == cudaSuccess ? GAS_OK : cuda_fail(e, "graph build");
}

gas_status device_csr_to_csc(cudaStream_t s, int32_t n, const uint32_t *cscPerm,
                             const uint32_t *csrPerm, int32_t *out) {
  if (n <= 0) return GAS_OK;
  uint32_t *inv = nullptr;
  cudaError_t e = cudaMallocAsync(&inv, sizeof(uint32_t) * n, s);
  if (e == cudaSuccess) {
    invert_kernel<<<grid_for(n), 256, 0, s>>>(cscPerm, n, inv);
    compose_kernel<<<grid_for(n), 256, 0, s>>>(inv, csrPerm, n, out);
    e = cudaGetLastError();
    cudaFreeAsync(inv, s);
  }
  return e == cudaSuccess ? GAS_OK : cuda_fail(e, "CSR to CSC edge map");
}

gas_status device_gather_bytes(cudaStream_t s, const void *dIn, const uint32_t *dPerm, int32_t n,
                               int32_t bytes, void *dOut) {
  if (n <= 0 || bytes <= 0) return GAS_OK;
  gather_bytes_kernel<<<grid_for(n), 256, 0, s>>>(reinterpret_cast<const unsigned char *>(dIn),
                                                  dPerm, n, bytes,
                                                  reinterpret_cast<unsigned char *>(dOut));
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? GAS_OK : cuda_fail(e, "edge data permutation");
}

gas_status device_scatter_bytes(cudaStream_t s, const void *dIn, const uint32_t *dPerm, int32_t n,
                                int32_t bytes, void *dOut) {
  if (n <= 0 || bytes <= 0) return GAS_OK;
  scatter_bytes_kernel<<<grid_for(n), 256, 0, s>>>(reinterpret_cast<const unsigned char *>(dIn),
                                                   dPerm, n, bytes,
                                                   reinterpret_cast<unsigned char *>(dOut));
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? GAS_OK : cuda_fail(e, "edge data un-permutation");
}

}  // namespace internal
}  // namespace gas
