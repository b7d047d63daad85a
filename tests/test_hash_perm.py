"""The keyed permutation of psc_hash.h (pivot order of the SCC drivers): a
bijection on [0, k), and feistel_inv undoes it, which the device pivot-order
scatter relies on (CPU only: the header compiled with g++)."""
import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
PROGRAM = r'''
#include "psc_hash.h"
#include <cstdio>
#include <vector>
int main() {
  using namespace psc;
  const uint64_t ks[] = {1, 2, 3, 4, 5, 17, 1000, 4095, 4096, 4097, 65535, 65536, 1000003, 3000017};
  const uint64_t seeds[] = {1, 7, 123456789};
  for (uint64_t k : ks)
    for (uint64_t seed : seeds) {
      FeistelKey f = feistel_key(k, seed);
      std::vector<char> seen(k, 0);
      for (uint64_t i = 0; i < k; i++) {
        const uint64_t j = feistel(f, i);
        if (j >= k || seen[j]) {
          std::printf("not a bijection: k=%llu\n", (unsigned long long)k);
          return 1;
        }
        seen[j] = 1;
        if (feistel_inv(f, j) != i) {
          std::printf("inverse fails: k=%llu i=%llu\n", (unsigned long long)k, (unsigned long long)i);
          return 1;
        }
      }
    }
  std::printf("ok\n");
  return 0;
}
'''


def test_feistel_inverse(tmp_path):
    src = tmp_path / "perm.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "perm"
    inc = ROOT / "parallel-strong-connectivity_gb300" / "csrc"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", str(inc), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout
