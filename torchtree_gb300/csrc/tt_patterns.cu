// Site-pattern compression on the host (torchtree/evolution/site_pattern.py:69-97):
// the distinct columns of a byte matrix (one row per taxon, one column per
// site or codon byte position) in lexicographic order of the column read
// top to bottom, with their counts.  This is the reference's
// sorted(Counter(zip(*sequences))) on bytes, done with column hashes to group
// equal columns and one lexicographic sort of the distinct ones.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/torchtree_gb300.h"
#include "tt_launch.h"

namespace {

uint64_t column_hash(const uint8_t *c, int64_t n) {
  uint64_t h = 0xcbf29ce484222325ull ^ uint64_t(n);
  int64_t i = 0;
  for (; i + 8 <= n; i += 8) {
    uint64_t w;
    std::memcpy(&w, c + i, 8);
    h = (h ^ w) * 0x100000001b3ull;
    h ^= h >> 29;
  }
  for (; i < n; ++i) h = (h ^ c[i]) * 0x100000001b3ull;
  return h;
}

template <typename F>
void parallel_for(int64_t n, F &&f) {
  const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  const int64_t per = (n + hw - 1) / hw;
  std::vector<std::thread> pool;
  for (unsigned t = 0; t < hw; ++t) {
    const int64_t a = t * per, b = std::min(n, a + per);
    if (a < b) pool.emplace_back([&f, a, b] { f(a, b); });
  }
  for (auto &th : pool) th.join();
}

}  // namespace

extern "C" int tt_compress_columns(const uint8_t *matrix, int64_t rows, int64_t sites, int64_t *n_patterns,
                                   int64_t *first_site, int64_t *counts, int64_t *site_pattern) {
  if (!matrix || !n_patterns || !first_site || !counts || rows < 1 || sites < 0)
    return tt::record_error(TT_ERR_INVALID_ARGUMENT, "tt_compress_columns: NULL argument or empty matrix");
  *n_patterns = 0;
  if (sites == 0) return TT_OK;
  // columns contiguous: col[s][r]
  std::vector<uint8_t> col(size_t(rows) * sites);
  parallel_for(sites, [&](int64_t a, int64_t b) {
    for (int64_t r = 0; r < rows; ++r) {
      const uint8_t *src = matrix + r * sites;
      for (int64_t s = a; s < b; ++s) col[size_t(s) * rows + r] = src[s];
    }
  });
  std::vector<uint64_t> hash(sites);
  parallel_for(sites, [&](int64_t a, int64_t b) {
    for (int64_t s = a; s < b; ++s) hash[s] = column_hash(&col[size_t(s) * rows], rows);
  });
  auto colp = [&](int64_t s) { return &col[size_t(s) * rows]; };
  // group equal columns: sort sites by (hash, bytes, site)
  std::vector<int64_t> order(sites);
  for (int64_t s = 0; s < sites; ++s) order[s] = s;
  std::sort(order.begin(), order.end(), [&](int64_t a, int64_t b) {
    if (hash[a] != hash[b]) return hash[a] < hash[b];
    const int c = std::memcmp(colp(a), colp(b), size_t(rows));
    return c != 0 ? c < 0 : a < b;
  });
  std::vector<int64_t> reps, rep_count, group_of(sites);
  for (int64_t i = 0; i < sites; ++i) {
    const int64_t s = order[i];
    if (i == 0 || hash[s] != hash[order[i - 1]] || std::memcmp(colp(s), colp(order[i - 1]), size_t(rows)) != 0) {
      reps.push_back(s);  // smallest site index of the group (ties sorted by index)
      rep_count.push_back(0);
    }
    rep_count.back() += 1;
    group_of[s] = int64_t(reps.size()) - 1;
  }
  // lexicographic order of the distinct columns
  std::vector<int64_t> g(reps.size());
  for (size_t i = 0; i < g.size(); ++i) g[i] = int64_t(i);
  std::sort(g.begin(), g.end(),
            [&](int64_t a, int64_t b) { return std::memcmp(colp(reps[a]), colp(reps[b]), size_t(rows)) < 0; });
  std::vector<int64_t> rank(g.size());
  for (size_t p = 0; p < g.size(); ++p) {
    rank[g[p]] = int64_t(p);
    first_site[p] = reps[g[p]];
    counts[p] = rep_count[g[p]];
  }
  if (site_pattern)
    for (int64_t s = 0; s < sites; ++s) site_pattern[s] = rank[group_of[s]];
  *n_patterns = int64_t(g.size());
  return TT_OK;
}
