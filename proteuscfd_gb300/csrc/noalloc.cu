// Residual norms without any device allocation.
//
// Who needs this: a host application that owns every byte of GPU memory
// (a pool allocator it hands out itself, a fixed memory budget per tenant,
// a solver loop that must not allocate once it runs) cannot let a library
// call cudaMalloc behind its back - an allocation there can fail
// unpredictably, fragment the pool, or stall the device at a bad moment.
// Such callers pass their own device buffers for the input and the output;
// the only other memory this entry point touches is a fixed scratch array
// compiled into the library.
//
// The scratch array below holds one row of six partial sums per block of
// 2048 nodes, for at most kMaxBlocks blocks: 16384 x 6 doubles = 768 KiB,
// resident on every GPU that loads the library until the process exits.
// That bounds the input at kMaxNodes = 33,554,432 nodes; larger inputs are
// rejected with PCFD_ERR_ARG.
//
// Every call shares the one array.  Each call overwrites the rows it uses
// before reading them, so nothing has to be cleared between calls, but two
// calls that run on the GPU at the same time (different streams, or
// different host threads) race on it: serialise them.
#include "../../include/pcfd.h"

#include <cuda_runtime.h>

#include <mutex>
#include <string>

namespace {

constexpr int kThreads = 256;
constexpr int kRowsPerThread = 8;
constexpr long long kRowsPerBlock = (long long)kThreads * kRowsPerThread;  // 2048 nodes
constexpr int kMaxBlocks = 16384;
constexpr long long kMaxNodes = kRowsPerBlock * kMaxBlocks;  // 33,554,432
constexpr int kMaxDevices = 64;

// the scratch: partial sums of b^2, six per block (total, then per equation)
static __device__ __align__(256) double g_norm_scratch[kMaxBlocks * 6];

// Device addresses of g_norm_scratch, looked up once per device.  In host
// code the array's name is only a stand-in for the symbol, not a device
// address, so a kernel must never be given it directly.
double* g_scratch_addr[kMaxDevices] = {nullptr};
std::mutex g_scratch_mu;

// Pass 1: block k sums b^2 over its 2048 rows (thread t takes rows t,
// t+256, ...) in a fixed order and writes its six sums to scratch row k.
__global__ void __launch_bounds__(kThreads) k_norm_partials(long long nnode, const double* __restrict__ b,
                                                            double* __restrict__ scratch) {
  __shared__ double red[kThreads / 32][6];
  double acc[6] = {0, 0, 0, 0, 0, 0};
  const long long base = (long long)blockIdx.x * kRowsPerBlock;
  for (int r = 0; r < kRowsPerThread; r++) {
    long long i = base + (long long)r * kThreads + threadIdx.x;
    if (i < nnode)
      for (int t = 0; t < 5; t++) {
        double v = b[i * 5 + t];
        acc[1 + t] += v * v;
      }
  }
  acc[0] = acc[1] + acc[2] + acc[3] + acc[4] + acc[5];
  for (int c = 0; c < 6; c++) {
    double v = acc[c];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][c] = v;
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    double v = 0.0;
    for (int w = 0; w < kThreads / 32; w++) v += red[w][threadIdx.x];
    scratch[(size_t)blockIdx.x * 6 + threadIdx.x] = v;
  }
}

// Pass 2: fixed-order sum of the block rows; resGlobal = sqrt(sum b^2) /
// (nnode*5) and per equation sqrt(sum b_j^2) / nnode, as ParallelL2Norm
// and StridedParallelL2Norm define them (ucs/parallel.h:121,162).
__global__ void k_norm_finish(int nblocks, long long nnode, const double* __restrict__ scratch,
                              double* __restrict__ norms) {
  int c = threadIdx.x;
  if (c >= 6) return;
  double v = 0.0;
  for (int k = 0; k < nblocks; k++) v += scratch[(size_t)k * 6 + c];
  norms[c] = (c == 0) ? sqrt(v) / ((double)nnode * 5.0) : sqrt(v) / (double)nnode;
}

}  // namespace

// defined in solver.cu: the text pcfd_last_error returns on this thread
void pcfd_set_last_error(const std::string& msg);

namespace {
int fail(int code, const std::string& msg) {
  pcfd_set_last_error(msg);
  return code;
}
}  // namespace

extern "C" {

// Declared in include/pcfd.h; see the comment there for the contract.
PCFD_API int pcfd_residual_norms_noalloc(const double* b, long long nnode, double* norms, void* stream) {
  if (!b || !norms) return fail(PCFD_ERR_ARG, "pcfd_residual_norms_noalloc: null device pointer");
  if (nnode <= 0) return fail(PCFD_ERR_ARG, "pcfd_residual_norms_noalloc: nnode must be positive");
  if (nnode > kMaxNodes)
    return fail(PCFD_ERR_ARG, "pcfd_residual_norms_noalloc: nnode " + std::to_string(nnode) +
                                  " exceeds the fixed scratch limit of " + std::to_string(kMaxNodes) + " nodes");
  // a capturing stream is refused before any other runtime call: the call
  // synchronizes the stream, which a capture cannot contain
  cudaStream_t st = (cudaStream_t)stream;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  cudaError_t e = cudaStreamIsCapturing(st, &cap);
  if (e != cudaSuccess) return fail(PCFD_ERR_CUDA, std::string("cudaStreamIsCapturing: ") + cudaGetErrorString(e));
  if (cap != cudaStreamCaptureStatusNone)
    return fail(PCFD_ERR_ARG, "pcfd_residual_norms_noalloc: the stream is capturing; the call synchronizes "
                              "the stream and cannot be captured");
  int dev = -1;
  e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(PCFD_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return fail(PCFD_ERR_ARG, "pcfd_residual_norms_noalloc: device id out of range");
  double* scratch;
  {
    // one-time set-up on this device (the current one): translate the
    // symbol to its device address
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_norm_scratch);
      if (e != cudaSuccess || !p)
        return fail(PCFD_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      g_scratch_addr[dev] = (double*)p;
    }
    scratch = g_scratch_addr[dev];
  }
  // the stream must belong to the current device, whose scratch address was
  // looked up above
  if (st) {
    int sdev = -1;
    e = cudaStreamGetDevice(st, &sdev);
    if (e != cudaSuccess) return fail(PCFD_ERR_ARG, std::string("cudaStreamGetDevice: ") + cudaGetErrorString(e));
    if (sdev != dev)
      return fail(PCFD_ERR_ARG, "pcfd_residual_norms_noalloc: stream belongs to device " + std::to_string(sdev) +
                                    ", the current device is " + std::to_string(dev));
  }
  const int nblocks = (int)((nnode + kRowsPerBlock - 1) / kRowsPerBlock);
  k_norm_partials<<<nblocks, kThreads, 0, st>>>(nnode, b, scratch);
  k_norm_finish<<<1, 32, 0, st>>>(nblocks, nnode, scratch, norms);
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(PCFD_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return fail(PCFD_ERR_CUDA, std::string("synchronize: ") + cudaGetErrorString(e));
  return PCFD_OK;
}

}  // extern "C"
