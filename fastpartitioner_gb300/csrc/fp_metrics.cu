// Metric evaluation on the device state: the six evaluators of
// shared/metric.cpp computed in one pass over the nets.
//
//   TV   = sum over nets of (parts - 1)               TV_Refined, metric.cpp:70-86
//   CN   = nets with more than one part               CN,         metric.cpp:3-14
//   TM   = distinct (part of source, other part) pairs  TM_scratch, metric.cpp:122-186
//   MSM  = max over parts of its distinct targets     MGM_scratch, metric.cpp:216-284
//   MSV  = max over parts of sum (parts - 1) of nets it is source of
//                                                     MGV_Scratch, metric.cpp:301-335
//   MSRV = max over parts of send + received          MGAV_Scratch, metric.cpp:353-391
//
// Layout: one warp per net (grid-stride); per-CTA shared histograms of send and
// received volume flushed once per CTA; the (source part, target part) message
// pairs set bits of a K x K bit matrix in global memory (K*K/8 bytes).  All
// arithmetic is integer and order-independent, hence exact.

#include "fp_device.cuh"
#include "../../include/fastpart.h"

#include <mutex>

namespace fp {

namespace {

struct MetricScratch {
  unsigned long long* acc;   // [0]=TV [1]=CN
  long long* send;           // K, send volume per part (MSV = MSRV send)
  long long* recv;           // K
  uint32_t* pairs;           // K*words bits
};

__global__ void metrics_nets_kernel(DevInstance I, MetricScratch M) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int K = I.K;
  const int words = (K + 31) >> 5;
  long long* send_s = reinterpret_cast<long long*>(smem_raw);
  long long* recv_s = send_s + K;
  for (int p = threadIdx.x; p < K; p += blockDim.x) { send_s[p] = 0; recv_s[p] = 0; }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int wpb = blockDim.x >> 5;
  unsigned long long tv = 0, cn = 0;
  for (int e = blockIdx.x * wpb + (threadIdx.x >> 5); e < I.noe; e += gridDim.x * wpb) {
    const int n = I.ep_len[e];
    const int s = (int)I.nptr[e];
    const int sp = I.part_vec[I.src[e]];
    if (lane == 0) {
      if (n > 0) tv += (unsigned long long)(n - 1);
      if (n > 1) cn++;
      if (n > 0) atomicAdd((unsigned long long*)&send_s[sp], (unsigned long long)(n - 1));
    }
    for (int j = lane; j < n; j += 32) {
      const int p = I.ep_part[s + j];
      if (p != sp) {
        atomicAdd((unsigned long long*)&recv_s[p], 1ull);
        atomicOr(&M.pairs[(size_t)sp * words + (p >> 5)], 1u << (p & 31));
      }
    }
  }
  if (lane == 0) {
    if (tv) atomicAdd(&M.acc[0], tv);
    if (cn) atomicAdd(&M.acc[1], cn);
  }
  __syncthreads();
  for (int p = threadIdx.x; p < K; p += blockDim.x) {
    if (send_s[p]) atomicAdd((unsigned long long*)&M.send[p], (unsigned long long)send_s[p]);
    if (recv_s[p]) atomicAdd((unsigned long long*)&M.recv[p], (unsigned long long)recv_s[p]);
  }
}

// One CTA: TM = popcount of the pair matrix, MSM = max row popcount,
// MSV = max send, MSRV = max send + recv.
__global__ void metrics_final_kernel(DevInstance I, MetricScratch M, long long* out) {
  __shared__ long long red[4][32];
  const int K = I.K;
  const int words = (K + 31) >> 5;
  long long tm = 0, msm = -1, msv = -1, msrv = -1;
  for (int p = threadIdx.x; p < K; p += blockDim.x) {
    long long row = 0;
    for (int x = 0; x < words; x++) row += __popc(M.pairs[(size_t)p * words + x]);
    tm += row;
    msm = row > msm ? row : msm;
    msv = M.send[p] > msv ? M.send[p] : msv;
    const long long sr = M.send[p] + M.recv[p];
    msrv = sr > msrv ? sr : msrv;
  }
  for (int off = 16; off; off >>= 1) {
    tm += __shfl_xor_sync(0xffffffffu, tm, off);
    msm = max(msm, __shfl_xor_sync(0xffffffffu, msm, off));
    msv = max(msv, __shfl_xor_sync(0xffffffffu, msv, off));
    msrv = max(msrv, __shfl_xor_sync(0xffffffffu, msrv, off));
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) { red[0][warp] = tm; red[1][warp] = msm; red[2][warp] = msv; red[3][warp] = msrv; }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nw = blockDim.x >> 5;
    for (int w = 1; w < nw; w++) {
      tm += red[0][w];
      msm = max(msm, red[1][w]);
      msv = max(msv, red[2][w]);
      msrv = max(msrv, red[3][w]);
    }
    out[0] = (long long)M.acc[0];
    out[1] = (long long)M.acc[1];
    out[2] = tm;
    out[3] = msm;
    out[4] = msv;
    out[5] = msrv;
  }
}

}  // namespace

size_t metrics_scratch_bytes(int K) {
  const size_t words = (size_t)(K + 31) / 32;
  return 64 + 2 * sizeof(long long) * (size_t)K + sizeof(uint32_t) * words * (size_t)K;
}

// `scratch` must hold metrics_scratch_bytes(K) bytes (zeroed here);
// `out` receives 6 values on the device.
cudaError_t launch_metrics(const DevInstance& I, void* scratch, long long* out, int num_sms, cudaStream_t st,
                           int* launches) {
  const int K = I.K;
  const size_t words = (size_t)(K + 31) / 32;
  MetricScratch M;
  unsigned char* b = static_cast<unsigned char*>(scratch);
  M.acc = reinterpret_cast<unsigned long long*>(b);
  M.send = reinterpret_cast<long long*>(b + 64);
  M.recv = M.send + K;
  M.pairs = reinterpret_cast<uint32_t*>(M.recv + K);
  cudaError_t err = cudaMemsetAsync(scratch, 0, 64 + 2 * sizeof(long long) * K + sizeof(uint32_t) * words * K, st);
  if (err != cudaSuccess) return err;
  const int threads = 256;
  const size_t smem = 2 * sizeof(long long) * (size_t)K;
  err = cudaFuncSetAttribute(metrics_nets_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err != cudaSuccess) return err;
  int per_sm = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, metrics_nets_kernel, threads, smem);
  if (per_sm < 1) per_sm = 1;
  long long want = ((long long)I.noe + (threads / 32) - 1) / (threads / 32);
  long long grid = (long long)num_sms * per_sm;
  if (grid > want) grid = want > 0 ? want : 1;
  metrics_nets_kernel<<<(int)grid, threads, smem, st>>>(I, M);
  metrics_final_kernel<<<1, 1024, 0, st>>>(I, M, out);
  if (launches) *launches = 2;
  return cudaGetLastError();
}


// ---- metric evaluation without allocation ---------------------------------
//
// fp_metrics_noalloc evaluates the six metrics of a refinement state that the
// caller keeps in its own device memory, with the scratch of the two kernels
// above taken from a fixed array in the library's device image instead of a
// cudaMalloc'ed buffer.  The kernels are checked variants: the state comes
// straight from the caller, so a part id or list length out of range is
// flagged (all six outputs -1) instead of indexing past the array.

namespace {

constexpr int kNoAllocMaxK = FP_NOALLOC_MAX_K;
constexpr size_t noalloc_bytes(int K) {
  return 64 + 2 * sizeof(long long) * (size_t)K + sizeof(uint32_t) * (size_t)((K + 31) / 32) * (size_t)K;
}
constexpr size_t kNoAllocBytes = noalloc_bytes(kNoAllocMaxK);   // 147,520 bytes

// Shared by every call on a device and kept until the process exits.
static __device__ __align__(256) unsigned char g_metrics_scratch[kNoAllocBytes];

__global__ void metrics_nets_checked_kernel(DevInstance I, MetricScratch M) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int K = I.K;
  const int words = (K + 31) >> 5;
  long long* send_s = reinterpret_cast<long long*>(smem_raw);
  long long* recv_s = send_s + K;
  for (int p = threadIdx.x; p < K; p += blockDim.x) { send_s[p] = 0; recv_s[p] = 0; }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int wpb = blockDim.x >> 5;
  unsigned long long tv = 0, cn = 0;
  bool bad = false;
  for (int e = blockIdx.x * wpb + (threadIdx.x >> 5); e < I.noe; e += gridDim.x * wpb) {
    const int n = I.ep_len[e];
    const uint32_t s0 = I.nptr[e], s1 = I.nptr[e + 1];
    const int sv = I.src[e];
    if (s1 < s0 || (long long)s1 > I.pins || (unsigned)sv >= (unsigned)I.nov) {
      bad = true;
      continue;
    }
    const int s = (int)s0;
    const int cap = (int)(s1 - s0);
    const int sp = I.part_vec[sv];
    if (n < 0 || n > cap || (unsigned)sp >= (unsigned)K) {
      bad = true;
      continue;
    }
    if (lane == 0) {
      if (n > 0) tv += (unsigned long long)(n - 1);
      if (n > 1) cn++;
      if (n > 0) atomicAdd((unsigned long long*)&send_s[sp], (unsigned long long)(n - 1));
    }
    for (int j = lane; j < n; j += 32) {
      const int p = I.ep_part[s + j];
      if ((unsigned)p >= (unsigned)K) {
        bad = true;
      } else if (p != sp) {
        atomicAdd((unsigned long long*)&recv_s[p], 1ull);
        atomicOr(&M.pairs[(size_t)sp * words + (p >> 5)], 1u << (p & 31));
      }
    }
  }
  if (bad) atomicOr(&M.acc[2], 1ull);
  if (lane == 0) {
    if (tv) atomicAdd(&M.acc[0], tv);
    if (cn) atomicAdd(&M.acc[1], cn);
  }
  __syncthreads();
  for (int p = threadIdx.x; p < K; p += blockDim.x) {
    if (send_s[p]) atomicAdd((unsigned long long*)&M.send[p], (unsigned long long)send_s[p]);
    if (recv_s[p]) atomicAdd((unsigned long long*)&M.recv[p], (unsigned long long)recv_s[p]);
  }
}

__global__ void metrics_final_checked_kernel(DevInstance I, MetricScratch M, long long* out) {
  __shared__ long long red[4][32];
  const int K = I.K;
  const int words = (K + 31) >> 5;
  long long tm = 0, msm = -1, msv = -1, msrv = -1;
  for (int p = threadIdx.x; p < K; p += blockDim.x) {
    long long row = 0;
    for (int x = 0; x < words; x++) row += __popc(M.pairs[(size_t)p * words + x]);
    tm += row;
    msm = row > msm ? row : msm;
    msv = M.send[p] > msv ? M.send[p] : msv;
    const long long sr = M.send[p] + M.recv[p];
    msrv = sr > msrv ? sr : msrv;
  }
  for (int off = 16; off; off >>= 1) {
    tm += __shfl_xor_sync(0xffffffffu, tm, off);
    msm = max(msm, __shfl_xor_sync(0xffffffffu, msm, off));
    msv = max(msv, __shfl_xor_sync(0xffffffffu, msv, off));
    msrv = max(msrv, __shfl_xor_sync(0xffffffffu, msrv, off));
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) { red[0][warp] = tm; red[1][warp] = msm; red[2][warp] = msv; red[3][warp] = msrv; }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nw = blockDim.x >> 5;
    for (int w = 1; w < nw; w++) {
      tm += red[0][w];
      msm = max(msm, red[1][w]);
      msv = max(msv, red[2][w]);
      msrv = max(msrv, red[3][w]);
    }
    const bool bad = M.acc[2] != 0;
    out[0] = bad ? -1 : (long long)M.acc[0];
    out[1] = bad ? -1 : (long long)M.acc[1];
    out[2] = bad ? -1 : tm;
    out[3] = bad ? -1 : msm;
    out[4] = bad ? -1 : msv;
    out[5] = bad ? -1 : msrv;
  }
}

// Device address of g_metrics_scratch and the SM count, per device, found on
// the first call made with that device current.
constexpr int kNoAllocMaxDevices = 64;
struct NoAllocDevice {
  unsigned char* scratch = nullptr;
  int num_sms = 0;
};
std::mutex g_noalloc_mu;
NoAllocDevice g_noalloc_dev[kNoAllocMaxDevices];

}  // namespace

}  // namespace fp

extern "C" int fp_metrics_noalloc(int32_t K, int32_t nov, int32_t noe, int64_t pins, const uint32_t* nptr,
                                  const int32_t* src, const int32_t* part_vec, const int32_t* ep_len,
                                  const int32_t* ep_part, int64_t* out, void* stream) {
  using namespace fp;
  if (K > kNoAllocMaxK) return FP_ERR_UNSUPPORTED;   // beyond the fixed scratch array
  if (K < 2 || nov <= 0 || noe < 0 || pins < 0 || pins >= (1ll << 31) || !out ||
      (noe > 0 && (!nptr || !src || !part_vec || !ep_len || !ep_part)))
    return FP_ERR_INVALID;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return FP_ERR_CUDA;
  if (dev < 0 || dev >= kNoAllocMaxDevices) return FP_ERR_UNSUPPORTED;
  NoAllocDevice nd;
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    NoAllocDevice& slot = g_noalloc_dev[dev];
    if (!slot.scratch) {
      // The array's name in host code is not a device address: ask the runtime.
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_metrics_scratch) != cudaSuccess || !p) return FP_ERR_CUDA;
      int sms = 0;
      if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1)
        return FP_ERR_CUDA;
      slot.scratch = static_cast<unsigned char*>(p);
      slot.num_sms = sms;
    }
    nd = slot;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  MetricScratch M;
  M.acc = reinterpret_cast<unsigned long long*>(nd.scratch);
  M.send = reinterpret_cast<long long*>(nd.scratch + 64);
  M.recv = M.send + K;
  M.pairs = reinterpret_cast<uint32_t*>(M.recv + K);
  // Everything the kernels accumulate into starts at zero on every call.
  cudaError_t err = cudaMemsetAsync(nd.scratch, 0, noalloc_bytes(K), st);
  if (err != cudaSuccess) return FP_ERR_CUDA;
  DevInstance I{};
  I.K = K;
  I.nov = nov;
  I.noe = noe;
  I.pins = pins;
  I.nptr = nptr;
  I.src = src;
  I.part_vec = const_cast<int*>(part_vec);
  I.ep_len = const_cast<int*>(ep_len);
  I.ep_part = const_cast<int*>(ep_part);
  const int threads = 256;
  const size_t smem = 2 * sizeof(long long) * (size_t)K;   // <= 16 KB for K <= 1024
  long long want = ((long long)noe + (threads / 32) - 1) / (threads / 32);
  long long grid = (long long)nd.num_sms * 4;
  if (grid > want) grid = want > 0 ? want : 1;
  // cudaLaunchKernelEx returns each launch's own status, so an error the
  // caller left pending is neither reported as this call's nor cleared.
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  err = cudaLaunchKernelEx(&cfg, metrics_nets_checked_kernel, I, M);
  if (err != cudaSuccess) return FP_ERR_CUDA;
  cfg.gridDim = dim3(1);
  cfg.blockDim = dim3(1024);
  cfg.dynamicSmemBytes = 0;
  err = cudaLaunchKernelEx(&cfg, metrics_final_checked_kernel, I, M, reinterpret_cast<long long*>(out));
  return err == cudaSuccess ? FP_OK : FP_ERR_CUDA;
}
