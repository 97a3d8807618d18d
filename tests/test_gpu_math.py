"""The step's own math routines on the GPU.

* The correctly rounded division by a known reciprocal
  (feriphys_gb300/csrc/fastdiv.cuh) returns exactly the IEEE quotient: for
  every one of the 2^32 float numerators with the divisors 3 and pi, and for
  2^30 random (numerator, divisor) pairs, also through the integration's
  grouped F/m (physics.cuh: div_mass) with signed zero numerators mixed in.
* The branch-free reciprocals (fastdiv.cuh) equal the IEEE 1/x: rcp_rn_fast
  for every float of magnitude [2^-124, 2^124), rcp_of_root and its packed
  form for the square root of every float.
* The packed face pair (face_pair.cuh) gives lane by lane the bits of the
  scalar face terms (physics.cuh) on 2^22 random quads.
* The corner angle atan2(y, x), y >= 0 (feriphys_gb300/csrc/angle.cuh) stays
  within 3 ulp of a double-precision atan2 rounded to f32 over 2^28 random
  (y, x) pairs spread over many binades and over the special operands, and
  its packed two-lane form gives the scalar form's bits.
"""
import ctypes as C
import os
import subprocess
import tempfile

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

KERNEL = r"""
#include <cstdint>
#include "angle.cuh"
#include "face_pair.cuh"
#include "fastdiv.cuh"
#include "physics.cuh"
using namespace fgb;
__device__ __forceinline__ bool same(float x, float y) {
  return (__float_as_uint(x) == __float_as_uint(y)) || (isnan(x) && isnan(y));
}
__global__ void all_numerators(float b, float y, unsigned long long* bad) {
  unsigned long long local = 0;
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < (1ull << 32);
       i += (unsigned long long)gridDim.x * blockDim.x) {
    const float a = __uint_as_float(unsigned(i));
    if (!same(div_known_rcp(a, b, y), __fdiv_rn(a, b))) ++local;
  }
  if (local) atomicAdd(bad, local);
}
__device__ __forceinline__ unsigned mix(unsigned long long x) {
  x ^= x >> 33; x *= 0xff51afd7ed558ccdULL; x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ULL; x ^= x >> 33;
  return unsigned(x);
}
__global__ void random_pairs(unsigned long long n, unsigned long long* bad) {
  unsigned long long local = 0;
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    const float a = __uint_as_float(mix(2 * i));
    const float b = __uint_as_float(mix(2 * i + 1));
    const float ref = __fdiv_rn(a, b);
    const float got = rcp_usable(b) ? div_known_rcp(a, b, __frcp_rn(b)) : __fdiv_rn(a, b);
    if (!same(got, ref)) ++local;
    // the integration's grouped form (physics.cuh: div_mass), also for signed
    // zero numerators, which it answers without the IEEE fallback
    const float az = (i & 15) == 3 ? ((i & 16) ? -0.0f : 0.0f) : a;
    const V3<float> F{az, a, -a};
    const V3<float> q = div_mass(F, b, mass_div(b));
    if (!same(q.x, __fdiv_rn(az, b)) || !same(q.y, ref) || !same(q.z, __fdiv_rn(-a, b))) ++local;
  }
  if (local) atomicAdd(bad, local);
}
// ulp distance of two finite floats of the same sign (order-preserving integers)
__device__ __forceinline__ long long ordered(float x) {
  const int i = __float_as_int(x);
  return i >= 0 ? (long long)i : -(long long)(i & 0x7fffffff);
}
__global__ void angles(unsigned long long n, unsigned long long* worst_ulp, unsigned long long* bad_pair,
                       unsigned long long* n_fast, float one) {
  unsigned long long worst = 0, badp = 0, fast = 0;
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    // y >= 0 and x of either sign, magnitudes over 2^-40 .. 2^40, with every 64th pair exactly special
    const unsigned ry = mix(3 * i), rx = mix(3 * i + 1), rs = mix(3 * i + 2);
    float y = __uint_as_float(0x2b800000u + ry % 0x28000000u);
    float x = __uint_as_float((rx & 0x80000000u) | (0x2b800000u + (rx >> 1) % 0x28000000u));
    switch (rs & 63) {
      case 0: y = 0.0f; break;
      case 1: x = 0.0f; break;
      case 2: x = -0.0f; break;
      case 3: y = x = 0.0f; break;
      case 4: x = __uint_as_float(0x7f800000u); break;
      case 5: y = __uint_as_float(0x7f800000u); break;
      case 6: x = -y; break;
      case 7: x = y; break;
      default: break;
    }
    const float got = angle_pos(y, x);
    const float ref = (float)atan2((double)y, (double)x);
    const long long d = ordered(got) - ordered(ref);
    const unsigned long long u = (unsigned long long)(d < 0 ? -d : d);
    if (u > worst) worst = u;
    if (angle_detail::in_range(y, x)) ++fast;
    // the packed form, lane 0 and lane 1 with different operands
    const float y2 = angle_pos(x < 0.0f ? -x : x, y);
    const float2 p = upk(angle_pos2(pk(y, x < 0.0f ? -x : x), pk(x, y), pk(one, one)));
    if (!same(p.x, got) || !same(p.y, y2)) ++badp;
  }
  atomicMax(worst_ulp, worst);
  if (badp) atomicAdd(bad_pair, badp);
  atomicAdd(n_fast, fast);
}
extern "C" int run_angles(unsigned long long n, unsigned long long* out) {
  unsigned long long* d;
  if (cudaMalloc(&d, 3 * sizeof(unsigned long long)) != cudaSuccess) return -1;
  cudaMemset(d, 0, 3 * sizeof(unsigned long long));
  angles<<<4096, 256>>>(n, d, d + 1, d + 2, 1.0f);
  if (cudaMemcpy(out, d, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost) != cudaSuccess) return -2;
  cudaFree(d);
  return 0;
}
// Packed face pairs against the scalar face terms of the general kernels:
// random cloth-like triangles (a unit-spaced corner set jittered, scaled
// over many binades), velocities (some exactly zero) and wind.
__device__ __forceinline__ float unit(unsigned r) { return (r >> 8) * (1.0f / 16777216.0f) * 2.0f - 1.0f; }
__global__ void face_pairs(unsigned long long n, unsigned long long* bad, float* first, float one) {
  unsigned long long badl = 0;
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    unsigned long long k = 40 * i;
    const float sc = exp2f(float(int(mix(k++) % 24u)) - 12.0f);
    V3<float> x[4], v[4];
    const float cx[4] = {0, 1, 0, 1}, cy[4] = {0, 0, 1, 1};
    for (int j = 0; j < 4; ++j) {
      x[j] = V3<float>{sc * (cx[j] + 0.3f * unit(mix(k++))), sc * (cy[j] + 0.3f * unit(mix(k++))),
                       (i & 7) == 0 ? 0.0f : sc * 0.3f * unit(mix(k++))};
      const bool still = (i & 15) == 1;
      v[j] = V3<float>{still ? 0.0f : 3.0f * unit(mix(k++)), still ? 0.0f : 3.0f * unit(mix(k++)),
                       still ? 0.0f : 3.0f * unit(mix(k++))};
    }
    const V3<float> wind{2.0f * unit(mix(k++)), 2.0f * unit(mix(k++)), 2.0f * unit(mix(k++))};
    const float ncd = -0.6f, ncl = -0.3f;
    // quad corners 00 = x[0], 01 = x[1], 10 = x[2], 11 = x[3]; A = (01, 10, 00), B = (01, 11, 10)
    float4 DA, DB;
    float2 wA, wB;
    face_terms2(pk3(x[1], x[1]), pk3(x[2], x[3]), pk3(x[0], x[2]), pk3(v[1], v[1]), pk3(v[2], v[3]),
                pk3(v[0], v[2]), pk3(wind, wind), ncd, ncl, one, DA, wA, DB, wB);
    const int tri[2][3] = {{1, 2, 0}, {1, 3, 2}};
    const float got[2][6] = {{DA.x, DA.y, DA.z, DA.w, wA.x, wA.y}, {DB.x, DB.y, DB.z, DB.w, wB.x, wB.y}};
    for (int f = 0; f < 2; ++f) {
      const V3<float> a = x[tri[f][0]], b = x[tri[f][1]], c = x[tri[f][2]];
      const V3<float> D = face_total_force<float>(a, b, c, v[tri[f][0]], v[tri[f][1]], v[tri[f][2]], wind, ncd, ncl);
      const float ref[6] = {D.x, D.y, D.z, face_corner_weight<float>(a, b, c, 0),
                            face_corner_weight<float>(a, b, c, 1), face_corner_weight<float>(a, b, c, 2)};
      for (int q = 0; q < 6; ++q)
        if (!same(got[f][q], ref[q])) {
          if (atomicAdd(bad, 1ull) == 0) {
            first[0] = float(i); first[1] = float(f); first[2] = float(q);
            first[3] = got[f][q]; first[4] = ref[q];
            for (int j = 0; j < 3; ++j) {
              first[5 + 3 * j] = x[tri[f][j]].x; first[6 + 3 * j] = x[tri[f][j]].y; first[7 + 3 * j] = x[tri[f][j]].z;
            }
          }
          ++badl;
          break;
        }
    }
  }
}
extern "C" int run_faces(unsigned long long n, unsigned long long* out, float* first) {
  unsigned long long* d;
  float* df;
  if (cudaMalloc(&d, sizeof(unsigned long long)) != cudaSuccess) return -1;
  if (cudaMalloc(&df, 16 * sizeof(float)) != cudaSuccess) return -1;
  cudaMemset(d, 0, sizeof(unsigned long long));
  cudaMemset(df, 0, 16 * sizeof(float));
  face_pairs<<<1024, 256>>>(n, d, df, 1.0f);
  if (cudaMemcpy(out, d, sizeof(unsigned long long), cudaMemcpyDeviceToHost) != cudaSuccess) return -2;
  cudaMemcpy(first, df, 16 * sizeof(float), cudaMemcpyDeviceToHost);
  cudaFree(d);
  cudaFree(df);
  return 0;
}
// The branch-free reciprocals: rcp_rn_fast for every float of magnitude
// [2^-124, 2^124), either sign; rcp_of_root (and its packed form, with a
// second root in the other lane) for the square root of every float.
__global__ void reciprocals(unsigned long long* bad_fast, unsigned long long* bad_root,
                            unsigned long long* bad_pair, unsigned long long* n_fast) {
  unsigned long long bf = 0, br = 0, bp = 0, nf = 0;
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < (1ull << 32);
       i += (unsigned long long)gridDim.x * blockDim.x) {
    const float x = __uint_as_float(unsigned(i));
    const unsigned e = (unsigned(i) >> 23) & 0xffu;
    if (e >= 3 && e <= 250) {
      ++nf;
      if (!same(rcp_rn_fast(x), __fdiv_rn(1.0f, x))) ++bf;
    }
    const float m = __fsqrt_rn(x), m2 = __fsqrt_rn(__uint_as_float(unsigned(i) ^ 0x00400000u));
    if (!same(rcp_of_root(m), __fdiv_rn(1.0f, m))) ++br;
    const float2 p = upk(rcp_of_root2(pk(m, m2)));
    if (!same(p.x, __fdiv_rn(1.0f, m)) || !same(p.y, __fdiv_rn(1.0f, m2))) ++bp;
  }
  if (bf) atomicAdd(bad_fast, bf);
  if (br) atomicAdd(bad_root, br);
  if (bp) atomicAdd(bad_pair, bp);
  atomicAdd(n_fast, nf);
}
extern "C" int run_reciprocals(unsigned long long* out) {
  unsigned long long* d;
  if (cudaMalloc(&d, 4 * sizeof(unsigned long long)) != cudaSuccess) return -1;
  cudaMemset(d, 0, 4 * sizeof(unsigned long long));
  reciprocals<<<4096, 256>>>(d, d + 1, d + 2, d + 3);
  if (cudaMemcpy(out, d, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost) != cudaSuccess) return -2;
  cudaFree(d);
  return 0;
}
extern "C" int run(float b, float y, unsigned long long n_random, unsigned long long* out) {
  unsigned long long* d;
  if (cudaMalloc(&d, 4 * sizeof(unsigned long long)) != cudaSuccess) return -1;
  cudaMemset(d, 0, 4 * sizeof(unsigned long long));
  all_numerators<<<4096, 256>>>(b, y, d);
  random_pairs<<<4096, 256>>>(n_random, d + 1);
  if (cudaMemcpy(out, d, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost) != cudaSuccess) return -2;
  cudaFree(d);
  return 0;
}
"""


@pytest.fixture(scope="module")
def divlib():
    d = tempfile.mkdtemp(prefix="fgb_div_")
    src = os.path.join(d, "div.cu")
    open(src, "w").write(KERNEL)
    lib = os.path.join(d, "libdiv.so")
    subprocess.check_call(["nvcc", "-O3", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a", "-fmad=false",
                           "-Xcompiler", "-fPIC", "-shared", "-I", os.path.join(ROOT, "feriphys_gb300", "csrc"),
                           "-o", lib, src])
    l = C.CDLL(lib)
    l.run.argtypes = [C.c_float, C.c_float, C.c_ulonglong, C.POINTER(C.c_ulonglong)]
    l.run_angles.argtypes = [C.c_ulonglong, C.POINTER(C.c_ulonglong)]
    l.run_faces.argtypes = [C.c_ulonglong, C.POINTER(C.c_ulonglong), C.POINTER(C.c_float)]
    l.run_reciprocals.argtypes = [C.POINTER(C.c_ulonglong)]
    return l


@pytest.mark.parametrize("b,y", [(3.0, 0.333333343267440796), (3.14159265358979323846, 0.318309873342514038)])
def test_division_exact(divlib, b, y):
    out = (C.c_ulonglong * 4)()
    assert divlib.run(b, y, 1 << 30, out) == 0
    assert out[0] == 0, "%d numerators differ from IEEE division by %r" % (out[0], b)
    assert out[1] == 0, "%d random pairs differ from IEEE division" % out[1]


def test_angle_accuracy_and_pairs(divlib):
    out = (C.c_ulonglong * 3)()
    n = 1 << 28
    assert divlib.run_angles(n, out) == 0
    print("angle: worst %d ulp, %d of %d on the fast path" % (out[0], out[2], n))
    assert out[0] <= 3, "angle_pos is %d ulp from atan2 in double" % out[0]
    assert out[1] == 0, "%d packed results differ from the scalar ones" % out[1]
    assert out[2] > n // 2


def test_face_pairs_match_scalar_faces(divlib):
    """The tiled kernel's packed face pair gives, lane by lane, the bits of
    the scalar face terms the general and untiled kernels use."""
    out = (C.c_ulonglong * 1)()
    first = (C.c_float * 16)()
    assert divlib.run_faces(1 << 22, out, first) == 0
    assert out[0] == 0, "%d faces differ; first: %s" % (out[0], list(first))


def test_reciprocals_exact(divlib):
    """rcp_rn_fast is the IEEE reciprocal on its whole stated range, and
    rcp_of_root (scalar and packed) is 1/x for every square root a float can
    have, zeros, infinity and NaN included."""
    out = (C.c_ulonglong * 4)()
    assert divlib.run_reciprocals(out) == 0
    assert out[0] == 0, "%d operands of rcp_rn_fast differ from 1/x" % out[0]
    assert out[1] == 0, "%d square roots where rcp_of_root differs from 1/x" % out[1]
    assert out[2] == 0, "%d square roots where the packed rcp_of_root2 differs from 1/x" % out[2]
    assert out[3] == 2 * 248 * (1 << 23), out[3]
