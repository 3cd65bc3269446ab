"""The float-float helpers of the mixed path's Poisson refinement
(csrc/tpm_ff.cuh), checked on the host: the header is compiled with g++
against a stand-in cuda_runtime.h for its bit-cast intrinsics, with FP
contraction off, and tests/ff_check.cpp checks the double split (2^-48 bound,
truncated high part, zero / tiny / overflow / inf / nan), the exact float to
double conversion, TwoSum's exactness, the bounds of the product, the sums
and the difference of close pairs, the reciprocal (2^-45 bound), the
integer part / fraction / half decision read from a double's bits, and the
index division by a multiply-high (csrc/tpm_index.cuh) against the integer
quotient."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "triplyperiodic-modified_gb300", "csrc")

SHIM = """#pragma once
#include <cmath>
#include <cstring>
#define __device__
#define __forceinline__ inline
struct float2 { float x, y; };
inline float2 make_float2(float a, float b) { return {a, b}; }
inline long long __double_as_longlong(double d) { long long r; std::memcpy(&r, &d, 8); return r; }
inline double __longlong_as_double(long long v) { double r; std::memcpy(&r, &v, 8); return r; }
inline float __uint_as_float(unsigned u) { float f; std::memcpy(&f, &u, 4); return f; }
inline unsigned __float_as_uint(float f) { unsigned u; std::memcpy(&u, &f, 4); return u; }
inline float __uint2float_rn(unsigned u) { return (float)u; }
inline int __clzll(long long x) { return __builtin_clzll((unsigned long long)x); }
inline float __frcp_rn(float x) { return 1.0f / x; }
inline unsigned __umulhi(unsigned a, unsigned b) { return (unsigned)(((unsigned long long)a * b) >> 32); }
"""


def test_ff_helpers(tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    (tmp_path / "cuda_runtime.h").write_text(SHIM)
    exe = tmp_path / "ff_check"
    subprocess.check_call([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", str(tmp_path),
                           "-I", CSRC, os.path.join(HERE, "ff_check.cpp"), "-o", str(exe)])
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
