// Launch-shape autotuner (mcfd_autotune).
//
// The kernels take their launch shapes from mcfd_handle::tune: the block size
// of the face-flux kernels and of the dt reductions, and the width (blocks per
// SM) of the persistent limiter grid.  The tuner times every candidate on the
// handle's own mesh and current solution with CUDA events on the handle's
// stream (one untimed launch, then the mean of several), keeps the fastest,
// and drops the captured step graph so the next mcfd_advance captures the new
// shapes.  With a cache path the choice is looked up first and otherwise
// written there, one JSON object per line keyed by scheme, degree, precision,
// solver, limiter and cell-count bucket.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/mcfd.h"
#include "handle.hpp"

namespace {

constexpr int kReps = 5;

std::string tune_key(const mcfd_handle *h) {
  std::ostringstream k;
  const char *schemes[] = {"dgsem", "fr", "modal"};
  k << schemes[h->opt.scheme < 0 || h->opt.scheme > 2 ? 0 : h->opt.scheme] << "|p" << h->mesh.p
    << "|" << (h->opt.precision == 1 ? "mixed" : "fp64") << "|r" << h->opt.riemann << "|l"
    << h->lim.kind << "|c2^" << (int)std::lround(std::log2((double)std::max<int64_t>(h->mesh.n_cells, 1)));
  return k.str();
}

int read_int(const std::string &line, const char *field, int fallback) {
  const std::string tag = std::string("\"") + field + "\": ";
  const size_t at = line.find(tag);
  if (at == std::string::npos) return fallback;
  return std::atoi(line.c_str() + at + tag.size());
}

bool load_cached(const char *path, const std::string &key, mcfd::Tune *t) {
  std::ifstream in(path);
  if (!in) return false;
  const std::string tag = "\"key\": \"" + key + "\"";
  std::string line;
  while (std::getline(in, line)) {
    if (line.find(tag) == std::string::npos) continue;
    // block sizes other than the tuner's own (a damaged file) keep the defaults:
    // the dt kernels' per-block words assume 128 to 512 threads
    const auto block = [](int v, int fallback) { return (v == 128 || v == 256 || v == 512) ? v : fallback; };
    t->face_block = block(read_int(line, "face_block", t->face_block), t->face_block);
    t->dt_block = block(read_int(line, "dt_block", t->dt_block), t->dt_block);
    t->limiter_blocks_per_sm = read_int(line, "limiter_blocks_per_sm", t->limiter_blocks_per_sm);
    return true;
  }
  return false;
}

void store_cached(const char *path, const std::string &key, const mcfd::Tune &t,
                  const std::string &timings) {
  std::vector<std::string> keep;
  {
    std::ifstream in(path);
    std::string line;
    const std::string tag = "\"key\": \"" + key + "\"";
    while (in && std::getline(in, line))
      if (!line.empty() && line.find(tag) == std::string::npos) keep.push_back(line);
  }
  std::ofstream out(path, std::ios::trunc);
  for (const std::string &l : keep) out << l << "\n";
  out << "{\"key\": \"" << key << "\", \"face_block\": " << t.face_block
      << ", \"dt_block\": " << t.dt_block << ", \"limiter_blocks_per_sm\": "
      << t.limiter_blocks_per_sm << ", \"ms\": {" << timings << "}}\n";
}

// Mean milliseconds of `launch` (after one untimed call) on the handle's stream.
template <class F>
float time_ms(mcfd_handle *h, F &&launch, cudaError_t *err) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  launch();
  cudaEventRecord(e0, h->stream);
  for (int r = 0; r < kReps; ++r) launch();
  cudaEventRecord(e1, h->stream);
  cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess && *err == cudaSuccess) *err = e;
  return ms / kReps;
}

}  // namespace

extern "C" int mcfd_autotune(mcfd_handle *h, const char *cache_path, int32_t *choice) {
  if (!h) return MCFD_ERR_ARGUMENT;
  cudaSetDevice(h->device);
  const std::string key = tune_key(h);
  mcfd::Tune t = h->tune;
  bool cached = cache_path && load_cached(cache_path, key, &t);
  cudaError_t err = cudaSuccess;
  if (!cached) {
    std::ostringstream timings;
    mcfd::Buffers &b = h->buf;
    h->launches += mcfd::launch_set_state(h, h->t_host, 0.0, 1e300, h->opt.cfl > 0 ? h->opt.cfl : 0.1, 1);
    // face kernels (on the current solution, with its trace when used)
    const int face_sizes[] = {128, 256, 512};
    float best = 1e30f;
    for (int bs : face_sizes) {
      h->tune.face_block = bs;
      if (h->use_trace && h->trace_for != b.u) h->launches += mcfd::launch_trace(h, b.u);
      const float ms = time_ms(h, [&] { h->launches += mcfd::launch_face_flux(h, b.u, 0.0); }, &err);
      timings << "\"face_" << bs << "\": " << ms << ", ";
      if (ms < best) { best = ms; t.face_block = bs; }
    }
    h->tune.face_block = t.face_block;
    // dt reductions
    best = 1e30f;
    for (int bs : face_sizes) {
      h->tune.dt_block = bs;
      const float ms = time_ms(h, [&] { h->launches += mcfd::launch_dt(h, b.u); }, &err);
      timings << "\"dt_" << bs << "\": " << ms << ", ";
      if (ms < best) { best = ms; t.dt_block = bs; }
    }
    h->tune.dt_block = t.dt_block;
    // persistent limiter grid, on a scratch copy of the solution
    if (h->lim.kind != 0) {
      unsigned long long troubled = 0;
      cudaStreamSynchronize(h->stream);
      cudaMemcpy(&troubled, h->lim.troubled, sizeof(troubled), cudaMemcpyDeviceToHost);
      const int widths[] = {4, 8, 16, 32};
      best = 1e30f;
      for (int w : widths) {
        h->tune.limiter_blocks_per_sm = w;
        cudaMemcpyAsync(b.res, b.u, sizeof(double) * h->mesh.column, cudaMemcpyDeviceToDevice, h->stream);
        const float ms = time_ms(h, [&] { h->launches += mcfd::launch_limiter(h, b.res); }, &err);
        timings << "\"limiter_" << w << "\": " << ms << ", ";
        if (ms < best) { best = ms; t.limiter_blocks_per_sm = w; }
      }
      cudaMemcpy(h->lim.troubled, &troubled, sizeof(troubled), cudaMemcpyHostToDevice);
    }
    std::string tm = timings.str();
    if (tm.size() >= 2) tm.resize(tm.size() - 2);
    if (err == cudaSuccess && cache_path) store_cached(cache_path, key, t, tm);
  }
  if (err != cudaSuccess) {
    h->err = std::string("autotune: ") + cudaGetErrorString(err);
    return MCFD_ERR_CUDA;
  }
  t.tuned = true;
  h->tune = t;
  mcfd::drop_graphs(h);
  if (choice) {
    choice[0] = t.face_block;
    choice[1] = t.dt_block;
    choice[2] = t.limiter_blocks_per_sm;
    choice[3] = cached ? 1 : 0;
  }
  return MCFD_OK;
}
