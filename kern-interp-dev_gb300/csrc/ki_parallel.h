// Host-side parallel loop over contiguous index ranges (std::thread).
#pragma once

#include <algorithm>
#include <thread>
#include <vector>

namespace ki {

// fn(part, lo, hi) over [0, n) split into contiguous ranges, in part order,
// on up to 16 threads (one part on the caller's thread below `min_items`
// items).  Returns the number of parts.  fn must only write state owned by
// its part.
inline int parallel_part_count(int n, int min_items = 4096) {
  const int hw = (int)std::thread::hardware_concurrency();
  return (n < min_items) ? 1 : std::max(1, std::min(16, hw));
}

template <typename Fn>
int parallel_parts(int n, Fn fn, int min_items = 4096) {
  const int T = parallel_part_count(n, min_items);
  if (T == 1) {
    fn(0, 0, n);
    return 1;
  }
  const int chunk = (n + T - 1) / T;
  std::vector<std::thread> th;
  for (int t = 1; t < T; t++) {
    const int lo = std::min(n, t * chunk), hi = std::min(n, lo + chunk);
    th.emplace_back(fn, t, lo, hi);
  }
  fn(0, 0, std::min(n, chunk));
  for (auto& x : th) x.join();
  return T;
}

// fn(lo, hi) over the same ranges.
template <typename Fn>
void parallel_ranges(int n, Fn fn, int min_items = 4096) {
  parallel_parts(n, [&](int, int lo, int hi) { fn(lo, hi); }, min_items);
}

}  // namespace ki
