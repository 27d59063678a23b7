"""CPU: the per-device context table (cubigfloat_gb300/csrc/fpa_devctx.h) that keys the
library's SM count and error word by the current device, compiled for the host with a fake
device query: each device gets its own entry, made once by the first call that finds it
current (also when several host threads race to make it), a failed initialisation is
retried, and device numbers outside the table are refused."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "cubigfloat_gb300", "csrc")

PROG = r"""
#include <atomic>
#include <cstdio>
#include <thread>
#include <vector>
#include "fpa_devctx.h"

struct Ctx { int sms; long err; };
static thread_local int current = 0;            // stand-in for cudaSetDevice / cudaGetDevice
static std::atomic<int> inits[64];
static bool fail_next = false;

static bool query(int &d) { d = current; return true; }
static bool init(int d, Ctx &v) {
  if (fail_next) { fail_next = false; return false; }
  inits[d]++;
  v.sms = 100 + d; v.err = 0x1000 + 16 * d;
  return true;
}

int main() {
  PerDevice<Ctx> table;
  Ctx c{};
  int bad = 0;
  // device 0, then 1, then 0 again: two entries, one init each
  current = 0; bad += !table.get(query, init, c) || c.sms != 100 || c.err != 0x1000;
  current = 1; bad += !table.get(query, init, c) || c.sms != 101 || c.err != 0x1010;
  current = 0; bad += !table.get(query, init, c) || c.sms != 100;
  bad += inits[0] != 1 || inits[1] != 1;
  // a failed initialisation leaves the entry unset and the next call retries it
  current = 5; fail_next = true;
  bad += table.get(query, init, c);
  bad += table.peek(5, c);
  bad += !table.get(query, init, c) || c.sms != 105 || inits[5] != 1;
  // outside the table
  current = 64; bad += table.get(query, init, c);
  current = -1; bad += table.get(query, init, c);
  // eight threads per device on devices 2 and 3 race to make their entries
  std::vector<std::thread> ts;
  std::atomic<int> wrong{0};
  for (int t = 0; t < 16; t++)
    ts.emplace_back([&, t] {
      current = 2 + (t & 1);
      Ctx v{};
      for (int k = 0; k < 1000; k++)
        if (!table.get(query, init, v) || v.sms != 100 + current) wrong++;
    });
  for (auto &t : ts) t.join();
  bad += wrong.load() != 0 || inits[2] != 1 || inits[3] != 1;
  printf("%d\n", bad);
  return bad != 0;
}
"""


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not installed")
def test_per_device_context(tmp_path):
    src = tmp_path / "devctx.cpp"
    src.write_text(PROG)
    exe = tmp_path / "devctx"
    subprocess.run(["g++", "-std=c++17", "-O1", "-pthread", "-I", CSRC, str(src), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
