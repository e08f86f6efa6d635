// Minimal glm stand-in used ONLY to compile the reference's own CUDA sources for the parity
// oracle (the reference's third_party/glm submodule is empty). Provides exactly what
// cuda_rasterizer/forward.{h,cu} and rasterizer_impl.cu use: vec3, vec4, column-major mat3 with
// column indexing, the scalar (diagonal) and 9-scalar (column by column) constructors,
// transpose, and the mat3 product (A*B)[i][j] = A[0][j]*B[i][0] + A[1][j]*B[i][1] + A[2][j]*B[i][2]
// summed left to right -- the textbook column-major product, restated from the maths.
#pragma once
#if defined(__CUDACC__)
#define FE_GLM_FN __host__ __device__ inline
#else
#define FE_GLM_FN inline
#endif

namespace glm {

struct vec3 {
  float x, y, z;
  FE_GLM_FN float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  FE_GLM_FN const float& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

struct vec4 {
  float x, y, z, w;
};

struct mat3 {
  vec3 col[3];
  FE_GLM_FN mat3() : col{{1.f, 0.f, 0.f}, {0.f, 1.f, 0.f}, {0.f, 0.f, 1.f}} {}
  FE_GLM_FN explicit mat3(float s) : col{{s, 0.f, 0.f}, {0.f, s, 0.f}, {0.f, 0.f, s}} {}
  FE_GLM_FN mat3(float a, float b, float c, float d, float e, float f, float g, float h, float k)
      : col{{a, b, c}, {d, e, f}, {g, h, k}} {}
  FE_GLM_FN vec3& operator[](int i) { return col[i]; }
  FE_GLM_FN const vec3& operator[](int i) const { return col[i]; }
};

FE_GLM_FN mat3 transpose(const mat3& m) {
  return mat3(m[0][0], m[1][0], m[2][0], m[0][1], m[1][1], m[2][1], m[0][2], m[1][2], m[2][2]);
}

FE_GLM_FN mat3 operator*(const mat3& a, const mat3& b) {
  mat3 r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) r[i][j] = a[0][j] * b[i][0] + a[1][j] * b[i][1] + a[2][j] * b[i][2];
  return r;
}

}  // namespace glm
