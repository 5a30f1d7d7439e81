// Self-check of the dataflow sweep's bounded waits: one task of a tiny
// synthetic front (32 rows, one right-hand side, valid buffers throughout)
// waits on a counter.  With `starve` nothing ever sets that counter, so the
// wait must run out, raise ST_TIMEOUT and let the kernel finish (the task
// then computes on the data it has, which is still inside its buffers); the
// device stays usable.  Without `starve` the counter is set beforehand and the
// task must pass with no error.  Changes no device setting.
#include <chrono>
#include <vector>

#include "../../include/sylver_gb300.h"
#include "numeric.hpp"

using namespace sylver_gb300;

extern "C" int sylver_gb300_dataflow_selftest(int starve, unsigned* status, double* seconds) {
  if (!status || !seconds) return SYLVER_ERROR_UNKNOWN;
  Runtime& rt = Runtime::get();
  if (!rt.init()) return SYLVER_ERROR_CUDA_UNKNOWN;
  try {
    prepare_solve_kernels<float>();
    const int n = 32;
    const cudaStream_t s = rt.stream;
    DevMem fr, scr, xs, ys, tt, ttoff, cnt, dfo, tasks, err, pm;
    std::vector<FrontDesc> hfr(1);
    hfr[0] = FrontDesc{};
    hfr[0].off = 0;
    hfr[0].m = n;
    hfr[0].n = n;
    hfr[0].ld = n;
    fr.upload(hfr, s);
    scr.upload(std::vector<int64_t>{0}, s);
    ttoff.upload(std::vector<int64_t>{0}, s);
    dfo.upload(std::vector<int2>{make_int2(1, 4)}, s);
    xs.ensure(n * sizeof(float));
    ys.ensure(n * sizeof(float));
    tt.ensure((size_t)LSOLVE_BW2 * 32 * sizeof(float));
    pm.ensure(sizeof(float) * 4);
    SG_CUDA(cudaMemsetAsync(xs.p, 0, n * sizeof(float), s));
    SG_CUDA(cudaMemsetAsync(ys.p, 0, n * sizeof(float), s));
    SG_CUDA(cudaMemsetAsync(tt.p, 0, tt.bytes, s));
    // counters: [0] ticket, [1] the waited one, [2] the task's own signal
    std::vector<int> hc{0, starve ? 0 : 1, 0, 0, 0};
    cnt.upload(hc, s);
    // z_0 = u_0 - t_0 on rows [0, 32), waiting for counter 1 >= 1
    std::vector<DfTask> ht{{DF_FIN_BWD, 0, 0, n, 0, 0, 1, 1, 1, -1, 0, 2, 0, 0, 0}};
    tasks.upload(ht, s);
    err.ensure(sizeof(unsigned));
    SG_CUDA(cudaMemsetAsync(err.p, 0, sizeof(unsigned), s));
    LsArgs<float, float> a{};
    a.fr = fr.as<FrontDesc>();
    a.nrhs = 1;
    a.n = n;
    a.scratch = xs.as<float>();
    a.ys = ys.as<float>();
    a.scr_off = scr.as<int64_t>();
    a.tt = tt.as<float>();
    a.dfc = cnt.as<int>();
    a.dfo = dfo.as<int2>();
    a.ttoff = ttoff.as<int64_t>();
    a.pmat = pm.as<float>();
    a.pmode = 1;
    SG_CUDA(cudaStreamSynchronize(s));
    const auto t0 = std::chrono::steady_clock::now();
    launch_chain(true, tasks.as<DfTask>(), 1, a, err.as<unsigned>(), s);
    unsigned h = 0;
    SG_CUDA(cudaMemcpyAsync(&h, err.p, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    SG_CUDA(cudaStreamSynchronize(s));
    *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    *status = h;
    return SYLVER_SUCCESS;
  } catch (const std::exception&) {
    return SYLVER_ERROR_CUDA_UNKNOWN;
  }
}
