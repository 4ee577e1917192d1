// Tile-shape autotuner of the face kernels (cells per block).
#include <cmath>
#include <map>
#include <mutex>
#include <tuple>

#include "atm_internal.h"

namespace atm {
namespace {
using Key = std::tuple<int, int, int, int, int, int, int>;  // dev fam k mode hg tsize ncb
std::mutex g_mu;
std::map<Key, int> g_tab;  // cells per block; -1 while being tuned

int log2_floor(int n) {
  int r = 0;
  while (n > 1) {
    n >>= 1;
    ++r;
  }
  return r;
}
}  // namespace

int tuned_cpb(bool tune, cudaStream_t st, int family, int k, int mode, bool hg, int tsize,
              int nc, bool idempotent, const std::function<cudaError_t(int)> &launch) {
  const int nq = 2 * k + 1, def = 128 / nq;
  if (nc < 2048) return def;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return def;
  const Key key{dev, family, k, mode, hg ? 1 : 0, tsize, log2_floor(nc)};
  {
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_tab.find(key);
    if (it != g_tab.end()) return it->second > 0 ? it->second : def;
    if (!tune || !idempotent) return def;
    g_tab[key] = -1;
  }
  const int cands[3] = {64 / nq, 128 / nq, 256 / nq};
  cudaEvent_t a = nullptr, b = nullptr;
  int best = def;
  float best_ms = INFINITY;
  if (cudaEventCreate(&a) == cudaSuccess && cudaEventCreate(&b) == cudaSuccess) {
    for (int cpb : cands) {
      if (cpb < 1) continue;
      if (launch(cpb) != cudaSuccess) {  // e.g. more shared memory than a block may have
        cudaGetLastError();
        continue;
      }
      cudaEventRecord(a, st);
      bool ok = true;
      for (int r = 0; r < 3 && ok; ++r) ok = launch(cpb) == cudaSuccess;
      cudaEventRecord(b, st);
      float ms = 0.0f;
      if (ok && cudaEventSynchronize(b) == cudaSuccess && cudaEventElapsedTime(&ms, a, b) == cudaSuccess &&
          ms < best_ms) {
        best_ms = ms;
        best = cpb;
      }
      cudaGetLastError();
    }
  }
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  std::lock_guard<std::mutex> lock(g_mu);
  g_tab[key] = best;
  return best;
}

int tune_table(int *out, int max_entries) {
  std::lock_guard<std::mutex> lock(g_mu);
  int n = 0;
  for (const auto &kv : g_tab) {
    if (kv.second <= 0) continue;
    if (out && n < max_entries) {
      int *o = out + 8L * n;
      o[0] = std::get<0>(kv.first);
      o[1] = std::get<1>(kv.first);
      o[2] = std::get<2>(kv.first);
      o[3] = std::get<3>(kv.first);
      o[4] = std::get<4>(kv.first);
      o[5] = std::get<5>(kv.first);
      o[6] = std::get<6>(kv.first);
      o[7] = kv.second;
    }
    ++n;
  }
  return n;
}

}  // namespace atm
