"""The served form's host work pool (CopyPool in cubigfloat_gb300/csrc/fpa_serve.cu), compiled
for the host from that source: many rounds of random sizes, back to back (the pattern that
could let a worker that wakes late run into the next round), every item run exactly once,
copies and zero fills landing where they should; and the same under ThreadSanitizer where a
TSan build can start."""
import os
import shutil
import subprocess

import pytest

from test_group_ops_host import tsan_starts

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "cubigfloat_gb300", "csrc", "fpa_serve.cu")

MAIN = r"""
#include <cstdio>
#include <random>
int main(int argc, char **argv) {
  const int rounds = argc > 1 ? atoi(argv[1]) : 20;
  CopyPool pool(6);
  std::mt19937 g(7);
  for (int r = 0; r < rounds; r++) {
    const size_t n = g() % 300;
    std::vector<std::atomic<int>> hits(n);
    for (auto &h : hits) h = 0;
    pool.for_each(n, [&](size_t i) { hits[i].fetch_add(1); });
    for (size_t i = 0; i < n; i++)
      if (hits[i].load() != 1) { printf("ERROR round %d item %zu ran %d times\n", r, i, hits[i].load()); return 1; }
    if (r % 50 == 0) {                       // copies: pieces of at most 1 MB, zero fills
      std::vector<Copy> cs;
      std::vector<std::vector<uint8_t>> src, dst;
      const int k = 1 + g() % 5;
      for (int c = 0; c < k; c++) {
        const size_t bytes = (g() % 3) * (1 << 20) + g() % 5000;
        src.emplace_back(bytes); dst.emplace_back(bytes, 0xAB);
        for (size_t b = 0; b < bytes; b++) src.back()[b] = (uint8_t)(b * 7 + c);
      }
      for (int c = 0; c < k; c++) cs.push_back({dst[c].data(), c == 0 ? nullptr : src[c].data(), dst[c].size()});
      pool.run(cs);
      for (int c = 0; c < k; c++)
        for (size_t b = 0; b < dst[c].size(); b++)
          if (dst[c][b] != (c == 0 ? 0 : src[c][b])) { printf("ERROR copy %d byte %zu\n", c, b); return 1; }
    }
  }
  printf("ok\n");
  return 0;
}
"""


def pool_source():
    s = open(SRC).read()
    body = s[s.index("struct Copy {"):s.index("struct Slot {")]
    body = body[:body.index("// device bytes one operation")] if "// device bytes one operation" in body else body
    head = ("#include <algorithm>\n#include <atomic>\n#include <condition_variable>\n#include <cstdint>\n"
            "#include <cstdlib>\n#include <cstring>\n#include <functional>\n#include <memory>\n#include <mutex>\n"
            "#include <thread>\n#include <vector>\n")
    return head + body + MAIN


def build(tmp, flags):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not found")
    src, exe = tmp / "pool.cpp", tmp / "pool"
    src.write_text(pool_source())
    r = subprocess.run([cxx, "-std=c++17", "-pthread", *flags, "-o", str(exe), str(src)], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return str(exe)


def test_pool_runs_every_item_once(tmp_path):
    exe = build(tmp_path, ["-O2"])
    out = subprocess.run([exe, "3000"], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0 and "ok" in out.stdout, out.stdout[-500:] + out.stderr[-500:]


def test_pool_has_no_races(tmp_path):
    try:
        exe = build(tmp_path, ["-O1", "-g", "-fsanitize=thread"])
    except AssertionError as e:
        pytest.skip("ThreadSanitizer build failed: " + str(e)[-300:])
    tsan_starts(exe)
    out = subprocess.run([exe, "300"], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0 and "ok" in out.stdout and "ThreadSanitizer" not in out.stderr, out.stderr[-3000:]
