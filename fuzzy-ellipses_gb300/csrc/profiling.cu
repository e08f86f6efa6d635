// profiling.cu -- pipe-throughput microbenchmarks that supply the FP32-FMA and MUFU (XU) peaks
// the blend's roofline is reported against (no measured copy of these peaks exists otherwise).
#include "fe_kernels.cuh"

namespace fe {

namespace {

constexpr int kChains = 8;

// Eight independent dependent FMA chains per thread: measures FFMA issue throughput.
__global__ void __launch_bounds__(256) peak_fma_kernel(float* out, int iters, float a, float b) {
  float x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) x[c] = threadIdx.x * 1e-3f + c;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = fmaf(x[c], a, b);
  }
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += x[c];
  if (s == 12345.678f) out[blockIdx.x] = s;  // keeps the chains live
}

// Eight independent ex2.approx chains per thread: measures MUFU.EX2 throughput.
__global__ void __launch_bounds__(256) peak_ex2_kernel(float* out, int iters) {
  float x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) x[c] = -1e-3f * (threadIdx.x + c);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = ex2_approx(x[c]) - 1.0f;
  }
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += x[c];
  if (s == 12345.678f) out[blockIdx.x] = s;
}

// Eight independent chains of packed fma.rn.f32x2 per thread (two FMAs per instruction).
__global__ void __launch_bounds__(256) peak_fma2_kernel(float* out, int iters, float a, float b) {
  f2_t x[kChains];
  const f2_t A = f2_pack(a, a), B = f2_pack(b, b);
#pragma unroll
  for (int c = 0; c < kChains; ++c) x[c] = f2_pack(threadIdx.x * 1e-3f + c, c * 0.5f);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = fma2(x[c], A, B);
  }
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < kChains; ++c) {
    float lo, hi;
    f2_unpack(x[c], lo, hi);
    s += lo + hi;
  }
  if (s == 12345.678f) out[blockIdx.x] = s;
}

// Failure-detection self-test: one block waits on an mbarrier that nothing ever arrives at,
// through the library's bounded mbarrier wait (globaltimer limit). The wait must give up after
// limit_ns and report FE_DEVERR_TIMEOUT, leaving the context usable.
__global__ void wait_selftest_kernel(unsigned long long limit_ns, uint32_t* status,
                                     unsigned long long* elapsed_ns) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  const unsigned long long t0 = global_timer_ns();
  const bool completed = mbar_wait_bounded(&bar, 0, limit_ns);
  __syncthreads();
  if (threadIdx.x == 0) {
    *status = completed ? 0u : FE_DEVERR_TIMEOUT;
    *elapsed_ns = global_timer_ns() - t0;
  }
}

}  // namespace

void launch_wait_selftest(unsigned long long limit_ns, uint32_t* status,
                          unsigned long long* elapsed_ns, cudaStream_t st) {
  wait_selftest_kernel<<<1, 32, 0, st>>>(limit_ns, status, elapsed_ns);
}

// Returns pipe operations per second: kind 0 = FFMA (one FMA per op), kind 1 = MUFU.EX2
// (the ex2 kernel also issues one FADD per op, on the FMA pipe), kind 2 = packed f32x2 FMA
// (counted as two FMAs per instruction).
double run_peak(int kind, int iters, float* scratch, cudaStream_t st) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 8, threads = 256;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  auto launch = [&]() {
    if (kind == 0) peak_fma_kernel<<<blocks, threads, 0, st>>>(scratch, iters, 0.999f, 1e-4f);
    else if (kind == 1) peak_ex2_kernel<<<blocks, threads, 0, st>>>(scratch, iters);
    else peak_fma2_kernel<<<blocks, threads, 0, st>>>(scratch, iters, 0.999f, 1e-4f);
  };
  launch();  // warm-up
  cudaEventRecord(e0, st);
  for (int r = 0; r < 5; ++r) launch();
  cudaEventRecord(e1, st);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const double ops = 5.0 * blocks * threads * (double)iters * kChains * (kind == 2 ? 2.0 : 1.0);
  return ms > 0.f ? ops / (ms * 1e-3) : 0.0;
}

}  // namespace fe
