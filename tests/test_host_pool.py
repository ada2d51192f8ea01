"""The host worker pool behind the library's parallel loops (ki_parallel.h):
every index of a range is visited exactly once, in contiguous parts; a loop
started from inside a pool task (the pool is busy) and loops started from
several threads at once fall back to their own threads instead of waiting;
a forked child does not use the parent's workers.  Compiled with g++ and run
on the host."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "kern-interp-dev_gb300", "csrc")

PROGRAM = r"""
#include "ki_parallel.h"
#include <atomic>
#include <cstdio>
#include <sys/wait.h>
#include <thread>
#include <vector>

static bool cover(int n) {
  std::vector<std::atomic<int>> seen(n);
  for (auto& s : seen) s = 0;
  int prev_hi = 0;
  std::vector<std::pair<int, int>> parts(16, {-1, -1});
  const int T = ki::parallel_parts(n, [&](int t, int lo, int hi) {
    parts[t] = {lo, hi};
    for (int i = lo; i < hi; i++) seen[i]++;
  }, 1);
  for (int i = 0; i < n; i++)
    if (seen[i] != 1) return false;
  for (int t = 0; t < T; t++) {   // contiguous, in part order
    if (parts[t].first != prev_hi && parts[t].first < parts[t].second) return false;
    if (parts[t].second > parts[t].first) prev_hi = parts[t].second;
  }
  return prev_hi == n || n == 0;
}

int main() {
  int bad = 0;
  for (int n : {0, 1, 7, 16, 17, 1000, 100003})
    if (!cover(n)) { std::printf("cover %d failed\n", n); bad++; }
  // nested: a loop inside a pool task
  std::atomic<long> sum{0};
  ki::parallel_ranges(64, [&](int lo, int hi) {
    for (int i = lo; i < hi; i++)
      ki::parallel_ranges(1000, [&](int a, int b) { sum += b - a; }, 1);
  }, 1);
  if (sum != 64L * 1000) { std::printf("nested sum %ld\n", (long)sum); bad++; }
  // concurrent callers
  std::atomic<long> tot{0};
  std::vector<std::thread> callers;
  for (int c = 0; c < 4; c++)
    callers.emplace_back([&] {
      for (int r = 0; r < 50; r++) ki::parallel_ranges(5000, [&](int a, int b) { tot += b - a; }, 1);
    });
  for (auto& t : callers) t.join();
  if (tot != 4L * 50 * 5000) { std::printf("concurrent total %ld\n", (long)tot); bad++; }
  // a forked child loops on its own threads
  const pid_t pid = fork();
  if (pid == 0) _exit(cover(4096) ? 0 : 3);
  int st = 0;
  waitpid(pid, &st, 0);
  if (!WIFEXITED(st) || WEXITSTATUS(st) != 0) { std::printf("forked child failed\n"); bad++; }
  std::printf(bad ? "FAIL\n" : "OK\n");
  return bad;
}
"""


def test_worker_pool(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    src = tmp_path / "pool.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "pool"
    subprocess.run([gxx, "-O2", "-std=c++17", "-pthread", "-I" + CSRC, str(src), "-o", str(exe)],
                   check=True, capture_output=True, text=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout + r.stderr
