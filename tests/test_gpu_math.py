"""The step's correctly rounded division by a known reciprocal
(feriphys_gb300/csrc/fastdiv.cuh) returns exactly the IEEE quotient.

Checked on the GPU for every one of the 2^32 float numerators with the two
constant divisors the step uses (3 for the mean face velocity, pi for the
corner-angle weights), and for 2^30 random (numerator, divisor) pairs as in
the F/m of the integration.
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
#include "fastdiv.cuh"
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
  }
  if (local) atomicAdd(bad, local);
}
extern "C" int run(float b, float y, unsigned long long n_random, unsigned long long* out) {
  unsigned long long* d;
  if (cudaMalloc(&d, 2 * sizeof(unsigned long long)) != cudaSuccess) return -1;
  cudaMemset(d, 0, 2 * sizeof(unsigned long long));
  all_numerators<<<4096, 256>>>(b, y, d);
  random_pairs<<<4096, 256>>>(n_random, d + 1);
  if (cudaMemcpy(out, d, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost) != cudaSuccess) return -2;
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
    return l


@pytest.mark.parametrize("b,y", [(3.0, 0.333333343267440796), (3.14159265358979323846, 0.318309873342514038)])
def test_division_exact(divlib, b, y):
    out = (C.c_ulonglong * 2)()
    assert divlib.run(b, y, 1 << 30, out) == 0
    assert out[0] == 0, "%d numerators differ from IEEE division by %r" % (out[0], b)
    assert out[1] == 0, "%d random pairs differ from IEEE division" % out[1]
