"""Integer helpers of the device pattern build, compiled for the host with nvcc
and checked on the CPU:

* FastDiv (sysmat.cuh): multiply-shift division by an invariant divisor, used
  for slot -> (element, local entry) in every pattern-build kernel, against
  integer division for divisors 1..300 and larger ones, with numerators below
  2^31 (slot numbers);
* pack32 / unpack32 (pack32.cuh): 32-bit packing of a column's (row, slot)
  keys, which must keep the 64-bit order and round-trip.
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "elfel.jl_gb300", "csrc")

PROGRAM = r"""
#include <cstdio>
#include <cstdint>
#include <vector>
#include <algorithm>
#include "pack32.cuh"
#include "sysmat.cuh"
using namespace elfel;

static uint64_t rng = 88172645463325252ull;
static uint64_t next() { rng ^= rng << 13; rng ^= rng >> 7; rng ^= rng << 17; return rng; }

int main() {
  long bad = 0, checked = 0;
  std::vector<uint32_t> ds;
  for (uint32_t d = 1; d <= 300; ++d) ds.push_back(d);
  for (uint32_t d : {1000u, 4096u, 65535u, 123457u, 1048583u, 1073741827u, 2147483647u}) ds.push_back(d);
  for (uint32_t d : ds) {
    FastDiv f;
    f.init(d);
    std::vector<uint32_t> ns = {0u, 1u, d - 1, d, d + 1, 2147483646u, 2147483647u};
    for (int k = 1; k < 64; ++k) {
      const uint64_t q = (uint64_t)k * d;
      for (int o = -1; o <= 1; ++o)
        if ((int64_t)q + o >= 0 && (int64_t)q + o < 2147483648ll) ns.push_back((uint32_t)(q + o));
    }
    for (int k = 0; k < 2000; ++k) ns.push_back((uint32_t)(next() & 0x7fffffffu));
    for (uint32_t n : ns) {
      if (n >= 2147483648u) continue;
      ++checked;
      if (f.div(n) != n / d) ++bad;
    }
  }
  std::printf("fastdiv %ld %ld\n", checked, bad);
  long pbad = 0, pchecked = 0;
  for (int trial = 0; trial < 2000; ++trial) {
    const int rb = (int)(next() % 20), sb = (int)(next() % (32 - rb));  // rb + sb <= 31
    const uint32_t rmin = (uint32_t)(next() % 3000000u), smin = (uint32_t)(next() % 60000000u);
    const uint32_t rspan = rb ? (uint32_t)((1ull << rb) - 1) : 0u, sspan = sb ? (uint32_t)((1ull << sb) - 1) : 0u;
    std::vector<uint64_t> keys;
    const int n = 2 + (int)(next() % 63);
    for (int i = 0; i < n; ++i) {
      const uint32_t r = rmin + (uint32_t)(rspan ? next() % ((uint64_t)rspan + 1) : 0);
      const uint32_t s = smin + (uint32_t)(sspan ? next() % ((uint64_t)sspan + 1) : 0);
      keys.push_back(((uint64_t)r << 32) | s);
    }
    keys.push_back(((uint64_t)rmin << 32) | smin);
    keys.push_back(((uint64_t)(rmin + rspan) << 32) | (smin + sspan));
    const Pack32 p{rmin, smin, sb};
    for (uint64_t a : keys) {
      ++pchecked;
      const uint32_t ka = pack32(a, p);
      if (unpack32(ka, p) != a || ka >= 0x80000000u) ++pbad;
      for (int j = 0; j < 4; ++j) {
        const uint64_t b = keys[next() % keys.size()];
        if ((a < b) != (ka < pack32(b, p))) ++pbad;
      }
    }
  }
  std::printf("pack32 %ld %ld\n", pchecked, pbad);
  return (bad || pbad) ? 1 : 0;
}
"""


def test_fastdiv_and_pack32_on_host(tmp_path):
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
    if nvcc is None:
        pytest.skip("nvcc not available")
    src = tmp_path / "pattern_math.cu"
    src.write_text(PROGRAM)
    exe = tmp_path / "pattern_math"
    include = os.path.join(os.path.dirname(CSRC), "..", "include")
    subprocess.run([nvcc, "-std=c++17", "-O2", "-I", CSRC, "-I", include, str(src), "-o", str(exe)],
                   check=True, capture_output=True, timeout=300)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    lines = dict(line.split(" ", 1) for line in out.stdout.strip().splitlines())
    checked, bad = map(int, lines["fastdiv"].split())
    assert checked > 500000 and bad == 0
    checked, bad = map(int, lines["pack32"].split())
    assert checked > 50000 and bad == 0
    assert out.returncode == 0
