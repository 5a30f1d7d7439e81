// Self-check of the tensor-core contribution-block update: a synthetic front
// (m = k + rows, ld = m) with random L21 and a zero contribution block goes
// through the same split + TMA + tcgen05 path the factorization uses; the
// result is compared with -L21 L21^T formed in FP64 on the host.
#include <cmath>
#include <random>
#include <vector>

#include "../../include/sylver_gb300.h"
#include "numeric.hpp"
#include "tc.hpp"

using namespace sylver_gb300;

extern "C" int sylver_gb300_tc_selfcheck(int rows, int k, double* max_rel_err) {
  if (rows < 1 || k < 1 || !max_rel_err) return SYLVER_ERROR_UNKNOWN;
  Runtime& rt = Runtime::get();
  if (!rt.init()) return SYLVER_ERROR_CUDA_UNKNOWN;
  try {
    const int m = k + rows, ld = (m + 3) / 4 * 4,
              pitch = (k + TC_KCHUNK - 1) / TC_KCHUNK * TC_KCHUNK;
    std::vector<float> h((size_t)ld * m, 0.f);
    std::mt19937 gen(7);
    std::uniform_real_distribution<float> U(-1.f, 1.f);
    for (int c = 0; c < k; ++c)
      for (int r = k; r < m; ++r) h[(size_t)c * ld + r] = U(gen);
    DevMem arena, planes, sp, tk, err;
    arena.ensure(h.size() * sizeof(float));
    SG_CUDA(cudaMemcpy(arena.p, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice));
    const int64_t pstride = ((int64_t)rows * pitch + 63) / 64 * 64;
    planes.ensure((size_t)3 * pstride * sizeof(uint16_t));
    std::vector<TcSplit> hs{{0, ld, m, k, k, 0, 0}};
    std::vector<TcTask> ht;
    for (int cj = 0; cj * 128 < rows; ++cj)
      for (int ri = cj; ri * 128 < rows; ++ri)
        ht.push_back({0, ld, k + ri * 128, k + cj * 128, m, m, ri * 128, cj * 128,
                      (k + TC_KCHUNK - 1) / TC_KCHUNK});
    sp.upload(hs, rt.stream);
    tk.upload(ht, rt.stream);
    err.ensure(sizeof(unsigned));
    SG_CUDA(cudaMemsetAsync(err.p, 0, sizeof(unsigned), rt.stream));
    CUtensorMap maps[3];
    for (int q = 0; q < 3; ++q)
      make_panel_map(&maps[q], planes.as<uint16_t>() + q * pstride, rows, pitch);
    launch_split_t(arena.as<float>(), sp.as<TcSplit>(), 1, (int64_t)rows,
                   planes.as<uint16_t>(), pstride, pitch, rt.stream);
    launch_update_tc(maps, arena.as<float>(), tk.as<TcTask>(), (int)ht.size(),
                     err.as<unsigned>(), rt.stream);
    unsigned herr = 0;
    SG_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof(unsigned), cudaMemcpyDeviceToHost, rt.stream));
    std::vector<float> out(h.size());
    SG_CUDA(cudaMemcpyAsync(out.data(), arena.p, h.size() * sizeof(float),
                            cudaMemcpyDeviceToHost, rt.stream));
    SG_CUDA(cudaStreamSynchronize(rt.stream));
    if (herr) return SYLVER_ERROR_CUDA_UNKNOWN;
    double worst = 0.0, scale = 0.0;
    for (int j = 0; j < rows; ++j)
      for (int i = j; i < rows; ++i) {
        double ref = 0.0;
        for (int c = 0; c < k; ++c)
          ref -= (double)h[(size_t)c * ld + k + i] * (double)h[(size_t)c * ld + k + j];
        double got = out[(size_t)(k + j) * ld + k + i];
        worst = std::max(worst, std::fabs(got - ref));
        scale = std::max(scale, std::fabs(ref));
      }
    *max_rel_err = scale > 0 ? worst / scale : worst;
    return SYLVER_SUCCESS;
  } catch (const std::exception&) {
    return SYLVER_ERROR_CUDA_UNKNOWN;
  }
}
