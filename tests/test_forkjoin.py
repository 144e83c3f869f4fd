"""The host fork-join pool of the path tracers (csrc/forkjoin.h), built into
a small program with g++: many short jobs, jobs posted before the workers
have started, an exception from one chunk.  No GPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROG = r"""
#include <cstdio>
#include <stdexcept>
#include <vector>
#include "forkjoin.h"
int main() {
  for (int nt : {1, 2, 4, 16}) {
    for (int rep = 0; rep < 50; rep++) {
      c2g::ForkJoin pool(nt);  // the first job may be posted before any worker runs
      std::vector<long> v(1000, 0);
      for (int j = 0; j < 200; j++)
        pool.run((long)v.size(), [&](long b, long e) { for (long i = b; i < e; i++) v[i] += i; });
      for (long i = 0; i < (long)v.size(); i++)
        if (v[i] != 200 * i) { std::printf("wrong sum at %ld\n", i); return 1; }
      bool threw = false;
      try {
        pool.run(1000, [&](long b, long e) { if (b <= 500 && 500 < e) throw std::runtime_error("x"); });
      } catch (const std::runtime_error &) { threw = true; }
      if (!threw) { std::printf("exception lost\n"); return 1; }
    }
  }
  std::printf("ok\n");
  return 0;
}
"""


@pytest.mark.skipif(shutil.which("g++") is None, reason="no g++")
def test_forkjoin_pool(tmp_path):
    src = tmp_path / "fj.cpp"
    src.write_text(PROG)
    exe = tmp_path / "fj"
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-pthread", "-I",
                           os.path.join(ROOT, "critic2_gb300", "csrc"), str(src), "-o", str(exe)])
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout + out.stderr
