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

template <class T>
__global__ void k_positions(int n, const Vec4<T>* __restrict__ pos, float* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const Vec4<T> P = pos[i];
  out[3 * size_t(i)] = float(P.x);
  out[3 * size_t(i) + 1] = float(P.y);
  out[3 * size_t(i) + 2] = float(P.z);
}

template <class T>
__global__ void k_set_pins(int n, const uint8_t* __restrict__ pinned, Vec4<T>* __restrict__ vel) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) vel[i].w = pinned[i] ? T(1) : T(0);
}

inline int nb(int n) { return (n + 255) / 256; }

}  // namespace

template <class T>
cudaError_t launch_unpack(int n, const float* pts, const uint8_t* pinned, void* pos, void* vel, void* force,
                          cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_unpack<T><<<nb(n), 256, 0, s>>>(n, pts, pinned, static_cast<Vec4<T>*>(pos), static_cast<Vec4<T>*>(vel),
                                    static_cast<Vec4<T>*>(force));
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_pack_f32(int n, const void* pos, const void* vel, const void* force, float* pts, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
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

}  // namespace fgb
