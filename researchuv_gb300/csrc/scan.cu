// Device-wide exclusive scan (counts -> offsets) used by the GPU assembly: per-block
// Kogge-Stone scans in shared memory, a recursive scan of the block totals, then a uniform
// add.  Integer arithmetic, so the result is exact and order-independent.
#include "common.cuh"

namespace ruv {
namespace {

constexpr int kScanBlock = 1024;

template <class T>
__global__ void k_scan_local(const T* __restrict__ in, int64_t* __restrict__ out, int64_t* __restrict__ sums,
                             int64_t n_plus1, int64_t n_in) {
  __shared__ int64_t warp_tot[32];
  int64_t i = (int64_t)blockIdx.x * kScanBlock + threadIdx.x;
  int64_t v = (i < n_in) ? (int64_t)in[i] : 0;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int64_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int64_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int64_t t = warp_tot[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int64_t y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    warp_tot[lane] = t;  // inclusive prefix of warp totals
  }
  __syncthreads();
  int64_t excl = x - v + (wid > 0 ? warp_tot[wid - 1] : 0);
  if (i < n_plus1) out[i] = excl;
  if (threadIdx.x == kScanBlock - 1) sums[blockIdx.x] = warp_tot[31];
}

__global__ void k_scan_add(int64_t* __restrict__ out, const int64_t* __restrict__ sums, int64_t n_plus1) {
  int64_t i = (int64_t)blockIdx.x * kScanBlock + threadIdx.x;
  if (i < n_plus1 && blockIdx.x > 0) out[i] += sums[blockIdx.x];
}

template <class T>
void scan_impl(const T* in, int64_t* out, int64_t n, Workspace& ws, cudaStream_t s, const std::string& tag,
               int depth) {
  int64_t n1 = n + 1;
  int64_t nb = (n1 + kScanBlock - 1) / kScanBlock;
  int64_t* sums = ws.get<int64_t>(tag + ".scan" + std::to_string(depth), nb + 1);
  k_scan_local<T><<<(unsigned)nb, kScanBlock, 0, s>>>(in, out, sums, n1, n);
  count_launches(1);
  RUV_LAUNCH_CHECK();
  if (nb > 1) {
    int64_t* sums_x = ws.get<int64_t>(tag + ".scanx" + std::to_string(depth), nb + 1);
    scan_impl<int64_t>(sums, sums_x, nb, ws, s, tag, depth + 1);
    k_scan_add<<<(unsigned)nb, kScanBlock, 0, s>>>(out, sums_x, n1);
    count_launches(1);
    RUV_LAUNCH_CHECK();
  }
}

}  // namespace

void exclusive_scan(const int32_t* in, int64_t* out, int64_t n, Workspace& ws, cudaStream_t s,
                    const std::string& tag) {
  scan_impl<int32_t>(in, out, n, ws, s, tag, 0);
}

void exclusive_scan_u8(const uint8_t* in, int64_t* out, int64_t n, Workspace& ws, cudaStream_t s,
                       const std::string& tag) {
  scan_impl<uint8_t>(in, out, n, ws, s, tag, 0);
}

}  // namespace ruv
