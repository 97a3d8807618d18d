// Conversion between the reference's Stateful point layout (10 f32 per point:
// mass, position, velocity, accumulated force -- springy_mesh.rs:242-255) and
// the device state (SoA: pos = {x, y, z, mass}, vel = {vx, vy, vz, pinned},
// force = {Fx, Fy, Fz, 0}).  Host buffers are copied raw into a device staging
// buffer and converted here, so a host round trip costs two DMA copies and two
// light kernels instead of a host-side transpose.
#include "devmath.cuh"
#include "state_io.h"

namespace fgb {

namespace {

template <class T>
__global__ void k_unpack(int n, const float* __restrict__ pts, const uint8_t* __restrict__ pinned,
                         Vec4<T>* __restrict__ pos, Vec4<T>* __restrict__ vel, Vec4<T>* __restrict__ force) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float* p = pts + 10 * size_t(i);
  pos[i] = make4<T>(V3<T>{T(p[1]), T(p[2]), T(p[3])}, T(p[0]));
  vel[i] = make4<T>(V3<T>{T(p[4]), T(p[5]), T(p[6])}, pinned[i] ? T(1) : T(0));
  if (force) force[i] = make4<T>(V3<T>{T(p[7]), T(p[8]), T(p[9])}, T(0));
}

template <class T, class O>
__global__ void k_pack(int n, const Vec4<T>* __restrict__ pos, const Vec4<T>* __restrict__ vel,
                       const Vec4<T>* __restrict__ force, O* __restrict__ pts) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const Vec4<T> P = pos[i], V = vel[i];
  O* o = pts + 10 * size_t(i);
  o[0] = O(P.w);
  o[1] = O(P.x); o[2] = O(P.y); o[3] = O(P.z);
  o[4] = O(V.x); o[5] = O(V.y); o[6] = O(V.z);
  if (force) {
    const Vec4<T> F = force[i];
    o[7] = O(F.x); o[8] = O(F.y); o[9] = O(F.z);
  } else {
    o[7] = O(0); o[8] = O(0); o[9] = O(0);
  }
}

// Positions as 3 f32 per vertex.  A block's 256 rows (3 KB) are assembled in
// shared memory and leave as 16-byte chunks when the destination allows it,
// so a pinned host buffer written across the host link gets whole lines.
template <class T>
__global__ void __launch_bounds__(256) k_positions(int n, const Vec4<T>* __restrict__ pos, float* __restrict__ out) {
  __shared__ __align__(16) float s[3 * 256];
  const int base = blockIdx.x * 256;
  const int i = base + threadIdx.x;
  if (i < n) {
    const Vec4<T> P = pos[i];
    s[3 * threadIdx.x] = float(P.x);
    s[3 * threadIdx.x + 1] = float(P.y);
    s[3 * threadIdx.x + 2] = float(P.z);
  }
  __syncthreads();
  const int rows = min(256, n - base);
  float* dst = out + 3 * size_t(base);
  if (rows == 256 && (reinterpret_cast<uintptr_t>(dst) & 15) == 0) {
    if (threadIdx.x < 192)
      reinterpret_cast<float4*>(dst)[threadIdx.x] = reinterpret_cast<const float4*>(s)[threadIdx.x];
  } else {
    for (int k = threadIdx.x; k < 3 * rows; k += 256) dst[k] = s[k];
  }
}

template <class T>
__global__ void k_set_pins(int n, const uint8_t* __restrict__ pinned, Vec4<T>* __restrict__ vel) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) vel[i].w = pinned[i] ? T(1) : T(0);
}

inline int nb(int n) { return (n + 255) / 256; }

// The same conversions for f32 state with the Stateful rows moved as
// coalesced 16-byte chunks through shared memory (256 points = 10 KB per
// block); the rows may sit in device memory or, mapped, in pinned host memory,
// which the kernel then reads or writes across the host link directly.  The
// row pointer must be 16-byte aligned.
constexpr int kIoBlock = 256;

__global__ void __launch_bounds__(kIoBlock) k_unpack_staged(int n, const float* __restrict__ pts,
                                                            const uint8_t* __restrict__ pinned,
                                                            float4* __restrict__ pos, float4* __restrict__ vel,
                                                            float4* __restrict__ force) {
  __shared__ __align__(16) float buf[10 * kIoBlock];
  const int first = blockIdx.x * kIoBlock;
  const int cnt = min(kIoBlock, n - first);
  const int nf = 10 * cnt;
  const float* src = pts + 10 * size_t(first);
  for (int k = threadIdx.x; k < nf / 4; k += kIoBlock)
    reinterpret_cast<float4*>(buf)[k] = reinterpret_cast<const float4*>(src)[k];
  for (int k = (nf / 4) * 4 + threadIdx.x; k < nf; k += kIoBlock) buf[k] = src[k];
  __syncthreads();
  const int t = threadIdx.x;
  if (t >= cnt) return;
  const float* p = buf + 10 * t;
  const int i = first + t;
  pos[i] = make_float4(p[1], p[2], p[3], p[0]);
  vel[i] = make_float4(p[4], p[5], p[6], pinned[i] ? 1.0f : 0.0f);
  if (force) force[i] = make_float4(p[7], p[8], p[9], 0.0f);
}

__global__ void __launch_bounds__(kIoBlock) k_pack_staged(int n, const float4* __restrict__ pos,
                                                          const float4* __restrict__ vel,
                                                          const float4* __restrict__ force, float* __restrict__ pts) {
  __shared__ __align__(16) float buf[10 * kIoBlock];
  const int first = blockIdx.x * kIoBlock;
  const int cnt = min(kIoBlock, n - first);
  const int t = threadIdx.x;
  if (t < cnt) {
    const int i = first + t;
    const float4 P = pos[i], V = vel[i];
    const float4 F = force ? force[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    float* o = buf + 10 * t;
    o[0] = P.w;
    o[1] = P.x; o[2] = P.y; o[3] = P.z;
    o[4] = V.x; o[5] = V.y; o[6] = V.z;
    o[7] = F.x; o[8] = F.y; o[9] = F.z;
  }
  __syncthreads();
  const int nf = 10 * cnt;
  float* dst = pts + 10 * size_t(first);
  for (int k = t; k < nf / 4; k += kIoBlock)
    reinterpret_cast<float4*>(dst)[k] = reinterpret_cast<const float4*>(buf)[k];
  for (int k = (nf / 4) * 4 + t; k < nf; k += kIoBlock) dst[k] = buf[k];
}

template <class T>
__global__ void k_render_vertices(int n, const Vec4<T>* __restrict__ pos, const int* __restrict__ face_off,
                                  const int* __restrict__ face_inc, const int4* __restrict__ face_vtx, float cr,
                                  float cg, float cb, float* __restrict__ out) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  V3<float> N{0.0f, 0.0f, 0.0f};
  for (int k = face_off[v]; k < face_off[v + 1]; ++k) {
    const int4 f = face_vtx[face_inc[k] >> 2];
    const Vec4<T> A = pos[f.x], B = pos[f.y], C = pos[f.z];
    const V3<float> a{float(A.x), float(A.y), float(A.z)};
    const V3<float> e1 = a - V3<float>{float(B.x), float(B.y), float(B.z)};
    const V3<float> e2 = a - V3<float>{float(C.x), float(C.y), float(C.z)};
    N = N + cross(e1, e2);
  }
  N = normalize(N);
  const Vec4<T> P = pos[v];
  float* o = out + 9 * size_t(v);
  o[0] = float(P.x);
  o[1] = float(P.y);
  o[2] = float(P.z);
  o[3] = cr;
  o[4] = cg;
  o[5] = cb;
  o[6] = N.x;
  o[7] = N.y;
  o[8] = N.z;
}

}  // namespace

template <class T>
cudaError_t launch_unpack(int n, const float* pts, const uint8_t* pinned, void* pos, void* vel, void* force,
                          cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  if (sizeof(T) == 4 && (reinterpret_cast<uintptr_t>(pts) & 15) == 0) {
    k_unpack_staged<<<(n + kIoBlock - 1) / kIoBlock, kIoBlock, 0, s>>>(
        n, pts, pinned, static_cast<float4*>(pos), static_cast<float4*>(vel), static_cast<float4*>(force));
    return cudaGetLastError();
  }
  k_unpack<T><<<nb(n), 256, 0, s>>>(n, pts, pinned, static_cast<Vec4<T>*>(pos), static_cast<Vec4<T>*>(vel),
                                    static_cast<Vec4<T>*>(force));
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_pack_f32(int n, const void* pos, const void* vel, const void* force, float* pts, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  if (sizeof(T) == 4 && (reinterpret_cast<uintptr_t>(pts) & 15) == 0) {
    k_pack_staged<<<(n + kIoBlock - 1) / kIoBlock, kIoBlock, 0, s>>>(
        n, static_cast<const float4*>(pos), static_cast<const float4*>(vel), static_cast<const float4*>(force), pts);
    return cudaGetLastError();
  }
  k_pack<T, float><<<nb(n), 256, 0, s>>>(n, static_cast<const Vec4<T>*>(pos), static_cast<const Vec4<T>*>(vel),
                                          static_cast<const Vec4<T>*>(force), pts);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_pack_f64(int n, const void* pos, const void* vel, const void* force, double* pts,
                            cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_pack<T, double><<<nb(n), 256, 0, s>>>(n, static_cast<const Vec4<T>*>(pos), static_cast<const Vec4<T>*>(vel),
                                           static_cast<const Vec4<T>*>(force), pts);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_positions(int n, const void* pos, float* out, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_positions<T><<<nb(n), 256, 0, s>>>(n, static_cast<const Vec4<T>*>(pos), out);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_set_pins(int n, const uint8_t* pinned, void* vel, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_set_pins<T><<<nb(n), 256, 0, s>>>(n, pinned, static_cast<Vec4<T>*>(vel));
  return cudaGetLastError();
}

#define FGB_IO_INST(T)                                                                                       \
  template cudaError_t launch_unpack<T>(int, const float*, const uint8_t*, void*, void*, void*, cudaStream_t); \
  template cudaError_t launch_pack_f32<T>(int, const void*, const void*, const void*, float*, cudaStream_t);   \
  template cudaError_t launch_pack_f64<T>(int, const void*, const void*, const void*, double*, cudaStream_t);  \
  template cudaError_t launch_positions<T>(int, const void*, float*, cudaStream_t);                           \
  template cudaError_t launch_set_pins<T>(int, const uint8_t*, void*, cudaStream_t);
FGB_IO_INST(float)
FGB_IO_INST(double)

template <class T>
cudaError_t launch_render_vertices(int n, const void* pos, const int* face_off, const int* face_inc,
                                   const int4* face_vtx, float r, float g, float b, float* out, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_render_vertices<T><<<(n + 255) / 256, 256, 0, s>>>(n, static_cast<const Vec4<T>*>(pos), face_off, face_inc,
                                                       face_vtx, r, g, b, out);
  return cudaGetLastError();
}

template cudaError_t launch_render_vertices<float>(int, const void*, const int*, const int*, const int4*, float,
                                                   float, float, float*, cudaStream_t);
template cudaError_t launch_render_vertices<double>(int, const void*, const int*, const int*, const int4*, float,
                                                    float, float, float*, cudaStream_t);

}  // namespace fgb
