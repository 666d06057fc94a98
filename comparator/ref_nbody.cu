// Timing comparator: the reference's GPU force kernel restated for GB300.
//
// The reference's GPU path (src/library/MDSystem.cu:21-153, launched by
// calculateNForces, :230-291) cannot be built on the GPU host: its sources
// are not there and it needs the downloaded helper_cuda.h and the removed
// cudaThread* calls.  This file restates its kernel algorithm so that the
// benchmark can report how that design performs on the same GB300 beside the
// library's kernels.  It is measurement infrastructure only: the library
// (liblj_gb300.so) neither links nor calls it.
//
// The algorithm, as the reference runs it:
//  * one thread per particle i, blocks of `block` threads; every block walks
//    all j in tiles of `block` float4 positions staged in shared memory, with
//    a barrier before and after each tile; the last tile holds
//    n - (tiles - 1) * block records (MDSystem.cu:73-103, :236-237);
//  * per pair (MDSystem.cu:21-56): r = x_i - x_j; minimum image
//    r -= periodic * L * lround(r / L) per component; pairs with r^2 <= 1e-6
//    are skipped (this also drops i = j); RDF bin min(floor(r^2 / dr2), 255)
//    counted with a global atomicAdd into the block's own 256 bins;
//    s = r^-2 (12 r^-12 - 6 r^-6); F_i += r s; w_i += r^-12 - r^-6;
//    virial_i += s r^2;
//  * per particle (MDSystem.cu:105-108, :131-136): F *= 4 (w unscaled),
//    virial *= 4/2/3, Force[i] = (F, w), and the virial is added to one
//    global float with atomicAdd;
//  * the per-block RDF bins are merged by a second kernel (MDSystem.cu:140-153).
// Here the constants the reference keeps in __constant__ symbols are kernel
// parameters, and the merge reads block g's bins at g * 256 (the reference's
// merge strides by its launch's block size, which is 256 only for 256-thread
// blocks).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

namespace {

constexpr int kRefBins = 256;

__device__ __forceinline__ void ref_pair(float4& acc, float4& me, const float4 other, int* hist, float L,
                                         float periodic, float dr2) {
  float rx = me.x - other.x, ry = me.y - other.y, rz = me.z - other.z;
  rx += -periodic * L * (float)lroundf(rx / L);
  ry += -periodic * L * (float)lroundf(ry / L);
  rz += -periodic * L * (float)lroundf(rz / L);
  const float d2 = rx * rx + ry * ry + rz * rz;
  if (d2 > 1e-6f) {
    const int bin = min(__float2int_rd(d2 / dr2), kRefBins - 1);
    if (hist) atomicAdd(hist + bin, 1);
    const float inv2 = 1.0f / d2;
    const float inv6 = inv2 * inv2 * inv2;
    const float s = inv2 * (12.0f * inv6 * inv6 - 6.0f * inv6);
    acc.x += rx * s;
    acc.y += ry * s;
    acc.z += rz * s;
    acc.w += inv6 * inv6 - inv6;
    me.w += s * d2;
  }
}

__global__ void k_ref_forces(const float4* __restrict__ pos, float4* __restrict__ force, int n, int last,
                             float L, float periodic, float dr2, int* rdf_blocks, float* pressure) {
  extern __shared__ float4 tile[];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  int* hist = rdf_blocks + (size_t)blockIdx.x * kRefBins;
  for (int b = threadIdx.x; b < kRefBins; b += blockDim.x) hist[b] = 0;
  __syncthreads();
  const int ii = i < n ? i : n - 1;
  if (i >= n) hist = nullptr;
  float4 me = pos[ii];
  me.w = 0.f;
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
  int t = 0;
  for (int j0 = 0; j0 < n - (int)blockDim.x; j0 += blockDim.x, ++t) {
    tile[threadIdx.x] = pos[t * blockDim.x + threadIdx.x];
    __syncthreads();
#pragma unroll 8
    for (int k = 0; k < (int)blockDim.x; ++k) ref_pair(acc, me, tile[k], hist, L, periodic, dr2);
    __syncthreads();
  }
  if ((int)threadIdx.x < last) tile[threadIdx.x] = pos[t * blockDim.x + threadIdx.x];
  __syncthreads();
#pragma unroll 8
  for (int k = 0; k < last; ++k) ref_pair(acc, me, tile[k], hist, L, periodic, dr2);
  __syncthreads();
  acc.x *= 4.f;
  acc.y *= 4.f;
  acc.z *= 4.f;
  me.w *= 4.0f / 2.0f / 3.0f;
  if (i < n) {
    force[i] = acc;
    atomicAdd(pressure, me.w);
  }
}

__global__ void k_ref_rdf_merge(const int* rdf_blocks, int blocks, int* rdf) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= kRefBins) return;
  int total = 0;
  for (int g = 0; g < blocks; ++g) total += rdf_blocks[(size_t)g * kRefBins + b];
  rdf[b] = total;
}

}  // namespace

extern "C" {

// Scratch bytes the comparator needs for n particles in blocks of `block`
// (the per-block RDF bins, the merged bins and the pressure word).
size_t ljref_scratch_bytes(int n, int block) {
  const int grid = (n + block - 1) / block;
  return sizeof(int) * (size_t)kRefBins * (grid + 1) + 16;
}

// One force evaluation in the reference's design, enqueued on `stream`:
// pos4/force4 are device float4[n]; scratch is ljref_scratch_bytes(n, block)
// device bytes; the merged 256 RDF bins and the pressure stay in scratch
// (ljref_results copies them out).  Returns a cudaError_t value.
int ljref_forces(const void* pos4, void* force4, int n, float L, int periodic, float dr2, int block, void* scratch,
                 void* stream) {
  if (n < 2 || block < 32 || block > 1024) return (int)cudaErrorInvalidValue;
  const int grid = (n + block - 1) / block;
  int last = n % block;
  if (last == 0) last = block;
  int* rdf_blocks = static_cast<int*>(scratch);
  int* rdf = rdf_blocks + (size_t)kRefBins * grid;
  float* pressure = reinterpret_cast<float*>(rdf + kRefBins);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemsetAsync(pressure, 0, sizeof(float), st);
  if (e != cudaSuccess) return (int)e;
  k_ref_forces<<<grid, block, sizeof(float4) * block, st>>>(static_cast<const float4*>(pos4),
                                                           static_cast<float4*>(force4), n, last, L,
                                                           periodic ? 1.0f : 0.0f, dr2, rdf_blocks, pressure);
  k_ref_rdf_merge<<<(kRefBins + 255) / 256, 256, 0, st>>>(rdf_blocks, grid, rdf);
  return (int)cudaGetLastError();
}

// Copies the merged RDF bins (256 ints) and the pressure sum after
// ljref_forces, synchronising `stream`.
int ljref_results(const void* scratch, int n, int block, int* rdf256, float* pressure, void* stream) {
  const int grid = (n + block - 1) / block;
  const int* rdf = static_cast<const int*>(scratch) + (size_t)kRefBins * grid;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemcpyAsync(rdf256, rdf, sizeof(int) * kRefBins, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(pressure, rdf + kRefBins, sizeof(float), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return (int)e;
}

}  // extern "C"
