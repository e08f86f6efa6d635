// ref_driver.cu -- runs the reference CUDA rasterizer's own binning kernels on a GPU to produce
// golden key-parity fixtures (TEST INFRASTRUCTURE ONLY; never linked into the product).
//
// The device code is the reference's, compiled from its sources by `make -C oracle ref` into
// oracle/_ref/*.cubin (forward.cu: preprocessCUDA; rasterizer_impl.cu: getGaussianTileKeys,
// getPerTileRanges). This host program replays the binning half of forwardJAX
// (cuda_rasterizer/rasterizer_impl.cu:205-302): preprocess -> inclusive scan -> key emission ->
// sort -> tile ranges. The scan and the sort run on the host: thrust's inclusive_scan of integers
// and its sort of unique 64-bit keys have exactly one possible result, so the host versions give
// the same output as the reference's thrust calls.
//
// usage: ref_driver <forward.cubin> <rasterizer_impl.cubin> <in.bin> <out.bin>
//   in.bin : int32 P, H, W; float n_std, tan_fovx, tan_fovy;
//            float means[3P], scales[3P], rots[4P], view[16], proj[16]
//   out.bin: int64 K; int32 radii[P]; float means2d[2P]; uint32 tiles_touched_inclusive[P];
//            uint64 keys_sorted[K]; uint32 ranges[2T]
#include <cuda.h>
#include <vector_types.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#define CK(x)                                                                  \
  do {                                                                         \
    CUresult r_ = (x);                                                         \
    if (r_ != CUDA_SUCCESS) {                                                  \
      const char* s_ = nullptr;                                                \
      cuGetErrorString(r_, &s_);                                               \
      std::fprintf(stderr, "%s failed: %s\n", #x, s_ ? s_ : "?");              \
      return 2;                                                                \
    }                                                                          \
  } while (0)

static bool find_fn(CUmodule mod, const char* needle, CUfunction* out) {
  unsigned int n = 0;
  if (cuModuleGetFunctionCount(&n, mod) != CUDA_SUCCESS) return false;
  std::vector<CUfunction> fns(n);
  if (cuModuleEnumerateFunctions(fns.data(), n, mod) != CUDA_SUCCESS) return false;
  for (CUfunction f : fns) {
    const char* name = nullptr;
    if (cuFuncGetName(&name, f) == CUDA_SUCCESS && name && std::strstr(name, needle)) {
      *out = f;
      return true;
    }
  }
  return false;
}

template <class T>
static bool rd(FILE* f, T* p, size_t n) { return std::fread(p, sizeof(T), n, f) == n; }

int main(int argc, char** argv) {
  if (argc != 5) {
    std::fprintf(stderr, "usage: %s forward.cubin rasterizer_impl.cubin in.bin out.bin\n", argv[0]);
    return 1;
  }
  FILE* fi = std::fopen(argv[3], "rb");
  if (!fi) return 1;
  int32_t P, H, W;
  float n_std, tan_fovx, tan_fovy;
  if (!rd(fi, &P, 1) || !rd(fi, &H, 1) || !rd(fi, &W, 1) || !rd(fi, &n_std, 1) ||
      !rd(fi, &tan_fovx, 1) || !rd(fi, &tan_fovy, 1))
    return 1;
  std::vector<float> means(3 * P), scales(3 * P), rots(4 * P), view(16), proj(16);
  if (!rd(fi, means.data(), means.size()) || !rd(fi, scales.data(), scales.size()) ||
      !rd(fi, rots.data(), rots.size()) || !rd(fi, view.data(), 16) || !rd(fi, proj.data(), 16))
    return 1;
  std::fclose(fi);

  CK(cuInit(0));
  CUdevice dev;
  CK(cuDeviceGet(&dev, 0));
  CUcontext ctx;
  CK(cuDevicePrimaryCtxRetain(&ctx, dev));
  CK(cuCtxSetCurrent(ctx));
  CUmodule mf, mi;
  CK(cuModuleLoad(&mf, argv[1]));
  CK(cuModuleLoad(&mi, argv[2]));
  CUfunction f_pre, f_keys, f_ranges;
  if (!find_fn(mf, "preprocessCUDA", &f_pre) || !find_fn(mi, "getGaussianTileKeys", &f_keys) ||
      !find_fn(mi, "getPerTileRanges", &f_ranges)) {
    std::fprintf(stderr, "reference kernels not found in the cubins\n");
    return 3;
  }

  const int gx = (W + 7) / 8, gy = (H + 7) / 8;
  const int64_t T = (int64_t)gx * gy;
  // rasterizer_impl.cu:205-206
  float focal_y = H / (2.0f * tan_fovy);
  float focal_x = W / (2.0f * tan_fovx);

  const size_t Pn = (size_t)std::max(P, 1);
  CUdeviceptr d_means, d_scales, d_rots, d_prcs, d_view, d_proj, d_radii, d_xy, d_cov, d_touched;
  CK(cuMemAlloc(&d_means, 12 * Pn));
  CK(cuMemAlloc(&d_scales, 12 * Pn));
  CK(cuMemAlloc(&d_rots, 16 * Pn));
  CK(cuMemAlloc(&d_prcs, 36 * Pn));
  CK(cuMemAlloc(&d_view, 64));
  CK(cuMemAlloc(&d_proj, 64));
  CK(cuMemAlloc(&d_radii, 4 * Pn));
  CK(cuMemAlloc(&d_xy, 8 * Pn));
  CK(cuMemAlloc(&d_cov, 24 * Pn));
  CK(cuMemAlloc(&d_touched, 4 * Pn));
  CK(cuMemcpyHtoD(d_means, means.data(), 12 * (size_t)P));
  CK(cuMemcpyHtoD(d_scales, scales.data(), 12 * (size_t)P));
  CK(cuMemcpyHtoD(d_rots, rots.data(), 16 * (size_t)P));
  CK(cuMemcpyHtoD(d_view, view.data(), 64));
  CK(cuMemcpyHtoD(d_proj, proj.data(), 64));
  CK(cuMemsetD8(d_radii, 0, 4 * Pn));
  CK(cuMemsetD8(d_xy, 0, 8 * Pn));
  CK(cuMemsetD8(d_touched, 0, 4 * Pn));

  dim3 grid(gx, gy, 1);
  if (P > 0) {
    void* args[] = {&P, &n_std, &d_means, &d_scales, &d_rots, &d_prcs, &d_view, &d_proj, &W, &H,
                    &tan_fovx, &tan_fovy, &focal_x, &focal_y, &d_radii, &d_xy, &d_cov, &grid,
                    &d_touched};
    CK(cuLaunchKernel(f_pre, (P + 255) / 256, 1, 1, 256, 1, 1, 0, nullptr, args, nullptr));
    CK(cuCtxSynchronize());
  }
  std::vector<uint32_t> touched(P);
  std::vector<int32_t> radii(P);
  std::vector<float> xy(2 * P);
  if (P > 0) {
    CK(cuMemcpyDtoH(touched.data(), d_touched, 4 * (size_t)P));
    CK(cuMemcpyDtoH(radii.data(), d_radii, 4 * (size_t)P));
    CK(cuMemcpyDtoH(xy.data(), d_xy, 8 * (size_t)P));
  }
  uint64_t acc = 0;
  for (int i = 0; i < P; ++i) {
    acc += touched[i];
    touched[i] = (uint32_t)acc;
  }
  const int64_t K = (int64_t)acc;
  std::vector<uint64_t> keys(K);
  std::vector<uint32_t> ranges(2 * T, 0);
  if (K > 0) {
    CK(cuMemcpyHtoD(d_touched, touched.data(), 4 * (size_t)P));
    CUdeviceptr d_keys, d_counts, d_ranges;
    CK(cuMemAlloc(&d_keys, 8 * (size_t)K));
    CK(cuMemAlloc(&d_counts, 4 * (size_t)T));
    CK(cuMemAlloc(&d_ranges, 8 * (size_t)T));
    CK(cuMemsetD8(d_counts, 0, 4 * (size_t)T));
    CK(cuMemsetD8(d_ranges, 0, 8 * (size_t)T));
    void* kargs[] = {&P, &d_xy, &d_touched, &d_keys, &d_counts, &d_radii, &grid};
    CK(cuLaunchKernel(f_keys, (P + 255) / 256, 1, 1, 256, 1, 1, 0, nullptr, kargs, nullptr));
    CK(cuCtxSynchronize());
    CK(cuMemcpyDtoH(keys.data(), d_keys, 8 * (size_t)K));
    std::sort(keys.begin(), keys.end());
    CK(cuMemcpyHtoD(d_keys, keys.data(), 8 * (size_t)K));
    int nk = (int)K;
    void* rargs[] = {&nk, &d_keys, &d_ranges};
    CK(cuLaunchKernel(f_ranges, (nk + 255) / 256, 1, 1, 256, 1, 1, 0, nullptr, rargs, nullptr));
    CK(cuCtxSynchronize());
    CK(cuMemcpyDtoH(ranges.data(), d_ranges, 8 * (size_t)T));
    cuMemFree(d_keys);
    cuMemFree(d_counts);
    cuMemFree(d_ranges);
  }
  FILE* fo = std::fopen(argv[4], "wb");
  if (!fo) return 1;
  std::fwrite(&K, 8, 1, fo);
  std::fwrite(radii.data(), 4, P, fo);
  std::fwrite(xy.data(), 4, 2 * (size_t)P, fo);
  std::fwrite(touched.data(), 4, P, fo);
  std::fwrite(keys.data(), 8, (size_t)K, fo);
  std::fwrite(ranges.data(), 4, 2 * (size_t)T, fo);
  std::fclose(fo);
  cuModuleUnload(mf);
  cuModuleUnload(mi);
  cuDevicePrimaryCtxRelease(dev);
  return 0;
}
