// thorin_ensemble.cu -- ensembles of disks advanced concurrently
// (include/thorin_ensemble.h): a pool of host threads over per-disk
// streams, and a wall-clock autotuner of the worker count and the order.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <string>
#include <thread>
#include <vector>
#include "thorin_kernels.cuh"
#include "../../include/thorin_ensemble.h"

extern thread_local std::string g_last_error;
long long thorin_disk_cells(const thorin_disk *d);

static std::vector<int> schedule(thorin_disk *const *disks, int n, int order)
{
  std::vector<int> idx(n);
  for (int k = 0; k < n; k++) idx[k] = k;
  if (order == THORIN_ORDER_LARGEST)
    std::stable_sort(idx.begin(), idx.end(),
                     [&](int a, int b) { return thorin_disk_cells(disks[a]) > thorin_disk_cells(disks[b]); });
  return idx;
}

extern "C" int thorin_ensemble_algogas(thorin_disk *const *disks, thorin_planets *const *systems, int n, int workers,
                                       int order, int *status)
{
  if (!disks || !systems || n < 1 || workers < 1 || (order != THORIN_ORDER_GIVEN && order != THORIN_ORDER_LARGEST)) {
    g_last_error = "ensemble: disks, systems, n >= 1, workers >= 1 and a known order required";
    return THORIN_ERR_ARG;
  }
  for (int k = 0; k < n; k++)
    if (!disks[k] || !systems[k]) {
      g_last_error = "ensemble: a disk or planetary system is missing";
      return THORIN_ERR_ARG;
    }
  const std::vector<int> idx = schedule(disks, n, order);
  std::vector<int> st(n, THORIN_OK);
  std::vector<std::string> err(n);
  int dev = 0;
  cudaGetDevice(&dev);
  std::atomic<int> next{0};
  auto work = [&]() {
    cudaSetDevice(dev);
    for (;;) {
      const int q = next.fetch_add(1);
      if (q >= n) break;
      const int k = idx[q];
      st[k] = thorin_gpu_algogas(disks[k], systems[k]);
      if (st[k] != THORIN_OK) err[k] = g_last_error;
    }
  };
  const int w = std::min(workers, n);
  std::vector<std::thread> pool;
  for (int t = 1; t < w; t++) pool.emplace_back(work);
  work();
  for (auto &t : pool) t.join();
  int first = THORIN_OK;
  for (int k = 0; k < n; k++) {
    if (status) status[k] = st[k];
    if (first == THORIN_OK && st[k] != THORIN_OK) {
      first = st[k];
      g_last_error = "ensemble disk " + std::to_string(k) + ": " + err[k];
    }
  }
  return first;
}

extern "C" int thorin_ensemble_tune(thorin_disk *const *disks, thorin_planets *const *systems, int n, int max_workers,
                                    int ndt, int *best_workers, int *best_order, double *best_ms_per_dt,
                                    double *sequential_ms_per_dt)
{
  if (!best_workers || !best_order || !best_ms_per_dt || max_workers < 1 || ndt < 1) {
    g_last_error = "ensemble_tune: output pointers, max_workers >= 1 and ndt >= 1 required";
    return THORIN_ERR_ARG;
  }
  std::vector<std::pair<int, int>> cand;
  for (int w = 1; w <= std::min(max_workers, n); w *= 2) {
    cand.push_back({w, THORIN_ORDER_GIVEN});
    if (w > 1) cand.push_back({w, THORIN_ORDER_LARGEST});
  }
  double best = 1e300;
  *best_workers = 1;
  *best_order = THORIN_ORDER_GIVEN;
  for (const auto &c : cand) {
    if (cudaDeviceSynchronize() != cudaSuccess) { g_last_error = "ensemble_tune: device error"; return THORIN_ERR_CUDA; }
    const auto t0 = std::chrono::steady_clock::now();
    for (int k = 0; k < ndt; k++) {
      const int s = thorin_ensemble_algogas(disks, systems, n, c.first, c.second, nullptr);
      if (s != THORIN_OK) return s;
    }
    if (cudaDeviceSynchronize() != cudaSuccess) { g_last_error = "ensemble_tune: device error"; return THORIN_ERR_CUDA; }
    const double ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count() / (double)ndt;
    if (c.first == 1 && sequential_ms_per_dt) *sequential_ms_per_dt = ms;
    if (ms < best) {
      best = ms;
      *best_workers = c.first;
      *best_order = c.second;
    }
  }
  *best_ms_per_dt = best;
  return THORIN_OK;
}
