"""The served form's resident store allocator (ResidentStore in
cubigfloat_gb300/csrc/fpa_serve.cu), compiled for the host from that source and driven by
random allocations and releases in random order: every block returned lies inside the store
and overlaps no live block, the free list never holds two adjacent blocks, free and live
bytes always add up to the capacity, a request that fits in no free block is refused
exactly when no free block is large enough, and releasing everything restores one block of
the whole capacity."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "cubigfloat_gb300", "csrc", "fpa_serve.cu")

MAIN = r"""
#include <cstdio>
#include <random>
#include <vector>
static int check(const ResidentStore &s, const std::map<uint64_t, uint64_t> &live, uint64_t cap) {
  uint64_t free_bytes = 0, end = 0;
  bool first = true;
  for (auto &b : s.free_blocks) {
    if (b.second == 0) return 1;                              // an empty free block
    if (!first && b.first <= end) return 2;                   // adjacent or overlapping free blocks
    if (b.first + b.second > cap) return 3;
    end = b.first + b.second; first = false; free_bytes += b.second;
    auto it = live.upper_bound(b.first);                      // a live block inside a free one
    if (it != live.begin() && std::prev(it)->first + std::prev(it)->second > b.first) return 4;
    if (it != live.end() && it->first < b.first + b.second) return 4;
  }
  uint64_t live_bytes = 0, lend = 0;
  first = true;
  for (auto &b : live) {
    if (!first && b.first < lend) return 5;                   // overlapping live blocks
    if (b.first + b.second > cap) return 6;
    lend = b.first + b.second; first = false; live_bytes += b.second;
  }
  return free_bytes + live_bytes == cap ? 0 : 7;
}
int main() {
  std::mt19937_64 g(11);
  for (int trial = 0; trial < 200; trial++) {
    const uint64_t cap = 256 * (1 + g() % 4096);
    ResidentStore s;
    s.reset(cap);
    std::map<uint64_t, uint64_t> live;
    for (int step = 0; step < 400; step++) {
      if (live.empty() || g() % 3) {
        const uint64_t bytes = 256 * (1 + g() % (1 + (g() % 2 ? 8 : cap / 256 / 4)));
        uint64_t largest = 0;
        for (auto &b : s.free_blocks) largest = std::max(largest, b.second);
        const uint64_t off = s.alloc(bytes);
        if (off == UINT64_MAX) {
          if (largest >= bytes) { printf("ERROR refused %llu with a free block of %llu\n", (unsigned long long)bytes, (unsigned long long)largest); return 1; }
        } else {
          if (largest < bytes) { printf("ERROR granted more than the largest free block\n"); return 1; }
          live.emplace(off, bytes);
        }
      } else {
        auto it = live.begin();
        std::advance(it, g() % live.size());
        s.release(it->first, it->second);
        live.erase(it);
      }
      const int e = check(s, live, cap);
      if (e) { printf("ERROR invariant %d at trial %d step %d\n", e, trial, step); return 1; }
    }
    while (!live.empty()) {
      auto it = live.begin();
      std::advance(it, g() % live.size());
      s.release(it->first, it->second);
      live.erase(it);
    }
    if (s.free_blocks.size() != 1 || s.free_blocks.begin()->first != 0 || s.free_blocks.begin()->second != cap) {
      printf("ERROR the store did not return to one block of its capacity\n");
      return 1;
    }
  }
  printf("ok\n");
  return 0;
}
"""


def store_source():
    s = open(SRC).read()
    body = s[s.index("struct ResidentStore {"):s.index("struct Slot {")]
    head = "#include <algorithm>\n#include <cstdint>\n#include <iterator>\n#include <map>\n"
    return head + body + MAIN


def test_resident_store_invariants(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not found")
    src, exe = tmp_path / "store.cpp", tmp_path / "store"
    src.write_text(store_source())
    r = subprocess.run([cxx, "-O2", "-std=c++17", "-o", str(exe), str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0 and out.stdout.strip().endswith("ok"), out.stdout[-2000:]
