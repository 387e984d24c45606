#include "Autotuner.hpp"

#include "DataUtils.hpp"
#include "GraphRepRunner.hpp"
#include "TuningTable.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <fstream>
#include <iomanip>
#include <limits>
#include <stdexcept>

namespace rajaperf {

namespace {

enum class Family { Map, Stream, Reduce, Scan, Hydro2D, Rows, Fdtd, Fixed };

Family familyOf(KernelID kid) {
  switch (kid) {
    case Stream_COPY: case Stream_MUL: case Stream_ADD: case Stream_TRIAD:
      return Family::Stream;
    case Stream_DOT: case Algorithm_REDUCE_SUM: case Lcals_FIRST_MIN:
      return Family::Reduce;
    case Algorithm_SCAN:
      return Family::Scan;
    case Lcals_HYDRO_2D:
      return Family::Hydro2D;
    case Polybench_JACOBI_2D:
      return Family::Rows;
    case Polybench_FDTD_2D:
      return Family::Fdtd;
    case Basic_DAXPY: case Basic_INIT3: case Basic_MULADDSUB: case Lcals_DIFF_PREDICT:
    case Lcals_EOS: case Lcals_FIRST_DIFF: case Lcals_HYDRO_1D: case Lcals_INT_PREDICT:
    case Lcals_PLANCKIAN: case Apps_DEL_DOT_VEC_2D: case Apps_ENERGY: case Apps_PRESSURE:
    case Apps_VOL3D:
      return Family::Map;
    default:
      return Family::Fixed;  // the other Polybench kernels: one shape each
  }
}

// Seconds per rep of `body` replayed from a graph of `reps` reps (min of 3).
double timeGraph(const KernelBase::RepBody& body, int64_t reps) {
  GraphRepRunner runner(reps);
  runner.capture(reps, body);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(runner.stream());
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  checkCuda(cudaEventCreate(&e0), "cudaEventCreate");
  checkCuda(cudaEventCreate(&e1), "cudaEventCreate");
  double best = std::numeric_limits<double>::max();
  try {
    runner.launch();  // warm-up replay
    for (int trial = 0; trial < 3; ++trial) {
      checkCuda(cudaEventRecord(e0, s), "cudaEventRecord");
      runner.launch();
      checkCuda(cudaEventRecord(e1, s), "cudaEventRecord");
      checkCuda(cudaEventSynchronize(e1), "cudaEventSynchronize");
      float ms = 0.f;
      checkCuda(cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime");
      best = std::min(best, static_cast<double>(ms) * 1e-3);
    }
  } catch (...) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    throw;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return best / static_cast<double>(reps);
}

}  // namespace

std::vector<b200_tune> autotuneCandidates(KernelID kid) {
  std::vector<b200_tune> out(1, b200_tune{});  // library default
  const Family f = familyOf(kid);
  if (f == Family::Scan) {  // default: pipelined; algo 1: one tile per CTA
    for (int items : {16, 32}) {
      b200_tune t{};
      t.algo = 1;
      t.items = items;
      out.push_back(t);
    }
    return out;
  }
  if (f == Family::Rows) {  // rows per thread of the column-segment stencil
    for (int items : {1, 2, 4, 8}) {
      b200_tune t{};
      t.items = items;
      out.push_back(t);
    }
    return out;
  }
  if (f == Family::Fdtd) {  // rows per tile of the one-launch step; algo 1: two launches
    for (int rows : {8, 32}) {
      b200_tune t{};
      t.tile_y = rows;
      out.push_back(t);
    }
    b200_tune t{};
    t.algo = 1;
    out.push_back(t);
    return out;
  }
  if (f == Family::Fixed) return out;
  const int blocks_h2d[] = {64, 128, 256};
  const int blocks[] = {128, 256, 512};
  for (int i = 0; i < 3; ++i) {
    if (f == Family::Hydro2D) {
      b200_tune t{};
      t.block_size = blocks_h2d[i];
      out.push_back(t);
      continue;
    }
    const int block = blocks[i];
    for (int items : {1, 2, 4, 8}) {
      if (f == Family::Reduce && items == 1) continue;
      for (int vec : {1, 2}) {
        if (vec == 2 && f != Family::Stream) continue;
        b200_tune t{};
        t.block_size = block;
        t.items = items;
        t.vec = (f == Family::Stream) ? vec : 0;
        out.push_back(t);
      }
    }
  }
  return out;
}

std::vector<AutotuneRecord> autotune(const std::vector<std::unique_ptr<KernelBase>>& kernels,
                                     const std::vector<std::vector<size_t>>& tunings) {
  std::vector<AutotuneRecord> recs;
  TuningTable& table = TuningTable::instance();
  for (size_t i = 0; i < kernels.size(); ++i) {
    KernelBase* k = kernels[i].get();
    const std::vector<b200_tune> cands = autotuneCandidates(k->getKernelID());
    if (cands.size() < 2) continue;
    // the default tuning's shape comes from the table, which the override feeds
    size_t tidx = k->getVariantTuningIndex(Base_GB300, k->getDefaultTuningName());
    if (tidx == k->getUnknownTuningIdx()) tidx = tunings[i].front();
    AutotuneRecord rec;
    rec.kernel = k->getName();
    rec.size = k->getActualProblemSize();
    rec.best_s = std::numeric_limits<double>::max();
    detail::resetDataInitCount();
    k->setUp(Base_GB300, tidx);
    try {
      k->prepareRun(tidx);
      int64_t reps = 0;
      for (size_t c = 0; c < cands.size(); ++c) {
        TuningTable::Entry e{rec.kernel, rec.size, rec.size, cands[c]};
        table.setOverride(e);
        double t = 0.0;
        try {
          KernelBase::RepBody body = k->makeRepBody(tidx);
          if (reps == 0) {
            // size the graph to about half a millisecond of device time
            const double t1 = timeGraph(body, 1);
            reps = static_cast<int64_t>(5e-4 / std::max(t1, 1e-7));
            reps = std::max<int64_t>(2, std::min<int64_t>(reps, 1000));
          }
          t = timeGraph(body, reps);
        } catch (const std::exception&) {
          checkCuda(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
          continue;  // shape rejected by the library
        }
        ++rec.candidates;
        if (c == 0) rec.default_s = t;
        if (t < rec.best_s) {
          rec.best_s = t;
          rec.best = cands[c];
        }
      }
      table.clearOverride();
      k->finishRun(tidx);
    } catch (...) {
      table.clearOverride();
      k->tearDown(Base_GB300, tidx);
      throw;
    }
    k->tearDown(Base_GB300, tidx);
    if (rec.candidates > 0) recs.push_back(rec);
  }
  return recs;
}

bool writeAutotuneTable(const std::vector<AutotuneRecord>& recs, const std::string& path) {
  std::ofstream f(path);
  if (!f) return false;
  f << "# Base_GB300 tuning table written by --autotune\n"
    << "# kernel min_size max_size key=value ...   (measured us/rep: best, default)\n";
  for (const AutotuneRecord& r : recs) {
    TuningTable::Entry e{r.kernel, r.size, r.size, r.best};
    f << TuningTable::format(e) << "  # " << std::fixed << std::setprecision(3)
      << r.best_s * 1e6 << " " << r.default_s * 1e6 << " us, " << r.candidates
      << " shapes\n";
  }
  return static_cast<bool>(f);
}

}  // namespace rajaperf
