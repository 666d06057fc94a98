// lj_render.cu -- headless particle image: a GPU splat of the positions into
// an RGBA8 buffer, the stand-in for the reference's OpenGL viewer
// (src/gui/MDSystemGL.cpp:32-160, which draws each particle as an orange
// (255, 127, 0) sphere of radius 0.5 sigma inside the box outline).
//
// Orthographic view along one axis, the viewer on the positive side of it.
// Pixel (i, j) of a W x H image covers [i, i+1) x [j, j+1) in units of L/W,
// L/H of the two other axes (i along the first, j along the second of the
// remaining axes in x, y, z order; image row r shows j = H - 1 - r).  A
// particle covers the pixels whose centres lie strictly inside its disc of
// radius R; among the particles covering a pixel the one whose sphere surface
// there, depth + sqrt(R^2 - d^2), is largest wins (ties: the larger index),
// via a 64-bit atomicMax on (orderable float32 surface depth, index).  The
// winner shades the pixel with the sphere normal's view component
// nz = sqrt(1 - d^2/R^2): colour * (0.3 + 0.7 nz), rounded half up.  All
// arithmetic is FP64 with separately rounded operations, which a CPU
// restatement repeats exactly.
#include <cuda_runtime.h>

#include <cstdint>

namespace ljgb {

namespace {

__device__ __forceinline__ uint32_t orderable(float f) {
  const uint32_t b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

struct RenderArgs {
  const double* x;  // component-major positions of the system
  int npad, p0, n;  // stride, first particle of the box, particles
  int axis;         // view axis (0, 1, 2)
  int W, H;
  double L, R;      // box side, particle radius (sigma units)
  unsigned long long* key;
};

__global__ void k_splat(RenderArgs a) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.n) return;
  const int ca = a.axis == 0 ? 1 : 0, cb = a.axis == 2 ? 1 : 2;
  const int p = a.p0 + k;
  const double xa = a.x[(size_t)ca * a.npad + p];
  const double xb = a.x[(size_t)cb * a.npad + p];
  const double depth = a.x[(size_t)a.axis * a.npad + p];
  const double sx = __ddiv_rn(a.L, (double)a.W), sy = __ddiv_rn(a.L, (double)a.H);  // sigma per pixel
  const double u = __ddiv_rn(xa, sx), v = __ddiv_rn(xb, sy);                           // centre in pixels
  const double R2 = __dmul_rn(a.R, a.R);
  const int i0 = max(0, (int)floor(__dsub_rn(u, __ddiv_rn(a.R, sx))) - 1);
  const int i1 = min(a.W - 1, (int)floor(__dadd_rn(u, __ddiv_rn(a.R, sx))) + 1);
  const int j0 = max(0, (int)floor(__dsub_rn(v, __ddiv_rn(a.R, sy))) - 1);
  const int j1 = min(a.H - 1, (int)floor(__dadd_rn(v, __ddiv_rn(a.R, sy))) + 1);
  for (int j = j0; j <= j1; ++j) {
    const double dy = __dmul_rn(__dsub_rn(__dadd_rn((double)j, 0.5), v), sy);
    const double dy2 = __dmul_rn(dy, dy);
    for (int i = i0; i <= i1; ++i) {
      const double dx = __dmul_rn(__dsub_rn(__dadd_rn((double)i, 0.5), u), sx);
      const double d2 = __dadd_rn(__dmul_rn(dx, dx), dy2);
      if (!(d2 < R2)) continue;
      const double surf = __dadd_rn(depth, __dsqrt_rn(__dsub_rn(R2, d2)));
      const unsigned long long key =
          ((unsigned long long)orderable((float)surf) << 32) | (unsigned long long)(unsigned)(k + 1);
      atomicMax(a.key + (size_t)j * a.W + i, key);
    }
  }
}

__global__ void k_shade(RenderArgs a, uint8_t* rgba) {
  const int pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= a.W * a.H) return;
  const int i = pix % a.W, j = pix / a.W;
  uint8_t* out = rgba + ((size_t)(a.H - 1 - j) * a.W + i) * 4;
  const unsigned long long key = a.key[pix];
  if (!key) {
    out[0] = out[1] = out[2] = 0;
    out[3] = 255;
    return;
  }
  const int k = (int)(key & 0xffffffffull) - 1;
  const int ca = a.axis == 0 ? 1 : 0, cb = a.axis == 2 ? 1 : 2;
  const int p = a.p0 + k;
  const double xa = a.x[(size_t)ca * a.npad + p];
  const double xb = a.x[(size_t)cb * a.npad + p];
  const double sx = __ddiv_rn(a.L, (double)a.W), sy = __ddiv_rn(a.L, (double)a.H);
  const double u = __ddiv_rn(xa, sx), v = __ddiv_rn(xb, sy);
  const double dx = __dmul_rn(__dsub_rn(__dadd_rn((double)i, 0.5), u), sx);
  const double dy = __dmul_rn(__dsub_rn(__dadd_rn((double)j, 0.5), v), sy);
  const double d2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
  const double nz = __dsqrt_rn(__dsub_rn(1.0, __ddiv_rn(d2, __dmul_rn(a.R, a.R))));
  const double f = __dadd_rn(0.3, __dmul_rn(0.7, nz));
  const double col[3] = {255.0, 127.0, 0.0};
  for (int c = 0; c < 3; ++c) out[c] = (uint8_t)(int)floor(__dadd_rn(__dmul_rn(col[c], f), 0.5));
  out[3] = 255;
}

}  // namespace

cudaError_t launch_render(const double* x, int npad, int p0, int n, int axis, int W, int H, double L, double R,
                          unsigned long long* key, uint8_t* rgba, cudaStream_t st) {
  RenderArgs a{x, npad, p0, n, axis, W, H, L, R, key};
  cudaError_t e = cudaMemsetAsync(key, 0, sizeof(unsigned long long) * (size_t)W * H, st);
  if (e != cudaSuccess) return e;
  k_splat<<<(n + 127) / 128, 128, 0, st>>>(a);
  k_shade<<<(W * H + 255) / 256, 256, 0, st>>>(a, rgba);
  return cudaGetLastError();
}

}  // namespace ljgb
