#include "Reports.hpp"

#include <algorithm>
#include <cmath>
#include <iomanip>
#include <limits>
#include <ostream>

namespace rajaperf {
namespace reports {

namespace {

const char* const kSep = " , ";
const char* const kKernelHead = "Kernel  ";

size_t kernelColumnWidth(const ReportData& d) {
  size_t w = std::string(kKernelHead).size();
  for (const KernelRow& k : d.kernels) w = std::max(w, k.name.size());
  return w + 1;
}

double entry(const Cell& c, Combiner m, int npasses) {
  switch (m) {
    case Combiner::Average: return c.tot_time / std::max(npasses, 1);
    case Combiner::Minimum: return c.min_time;
    case Combiner::Maximum: return c.max_time;
  }
  return 0.0;
}

// The shared layout of the timing and speedup CSVs: a title line (padded
// with one separator per column), a variant line, a tuning line, then one
// row per kernel; values right-aligned in columns as wide as the widest of
// their variant name, tuning name and prec + 2.
template <typename Value>
void writeCSV(std::ostream& os, const ReportData& d, const std::string& title, size_t prec,
              Value value) {
  const size_t kw = kernelColumnWidth(d);
  std::vector<std::vector<size_t>> colw(d.variants.size());
  for (size_t v = 0; v < d.variants.size(); ++v) {
    const size_t vw = std::max(prec + 2, d.variants[v].size());
    for (const std::string& t : d.tunings[v]) colw[v].push_back(std::max(vw, t.size()));
  }
  os << title;
  for (size_t v = 0; v < d.variants.size(); ++v)
    for (size_t t = 0; t < d.tunings[v].size(); ++t) os << kSep;
  os << "\n";
  os << std::left << std::setw(kw) << kKernelHead;
  for (size_t v = 0; v < d.variants.size(); ++v)
    for (size_t t = 0; t < d.tunings[v].size(); ++t)
      os << kSep << std::left << std::setw(colw[v][t]) << d.variants[v];
  os << "\n";
  os << std::left << std::setw(kw) << kKernelHead;
  for (size_t v = 0; v < d.variants.size(); ++v)
    for (size_t t = 0; t < d.tunings[v].size(); ++t)
      os << kSep << std::left << std::setw(colw[v][t]) << d.tunings[v][t];
  os << "\n";
  for (const KernelRow& k : d.kernels) {
    os << std::left << std::setw(kw) << k.name;
    for (size_t v = 0; v < d.variants.size(); ++v) {
      for (size_t t = 0; t < d.tunings[v].size(); ++t) {
        os << kSep << std::right << std::setw(colw[v][t]);
        double x = 0.0;
        if (!value(k, v, t, &x)) {
          os << "Not run";
        } else {
          os << std::setprecision(prec) << std::fixed << x;
        }
      }
    }
    os << "\n";
  }
  os.unsetf(std::ios::floatfield);
  os.flush();
}

const char* titlePrefix(Combiner c) {
  switch (c) {
    case Combiner::Average: return "Mean ";
    case Combiner::Minimum: return "Min ";
    case Combiner::Maximum: return "Max ";
  }
  return "";
}

}  // namespace

const char* combinerName(Combiner c) {
  switch (c) {
    case Combiner::Average: return "Average";
    case Combiner::Minimum: return "Minimum";
    case Combiner::Maximum: return "Maximum";
  }
  return "";
}

void writeTimingReport(std::ostream& os, const ReportData& d, Combiner c) {
  writeCSV(os, d, std::string(titlePrefix(c)) + "Runtime Report (sec.) ", 6,
           [&](const KernelRow& k, size_t v, size_t t, double* out) {
             const Cell& cell = k.cells[v][t];
             if (!cell.defined) return false;
             *out = entry(cell, c, d.npasses);
             return true;
           });
}

void writeSpeedupReport(std::ostream& os, const ReportData& d, Combiner c) {
  if (d.reference_variant < 0) return;
  const size_t rv = static_cast<size_t>(d.reference_variant);
  const std::string title = std::string(titlePrefix(c)) +
                            "Speedup Report (T_ref/T_var): ref var = " + d.variants[rv] + " ";
  // the reference column is the reference variant's first tuning
  writeCSV(os, d, title, 3, [&](const KernelRow& k, size_t v, size_t t, double* out) {
    if (k.cells[rv].empty()) return false;
    const Cell& ref = k.cells[rv][0];
    const Cell& cell = k.cells[v][t];
    if (!ref.defined || !cell.defined) return false;
    const double tv = entry(cell, c, d.npasses);
    *out = tv > 0.0 ? entry(ref, c, d.npasses) / tv : 0.0;
    return true;
  });
}

void writeChecksumReport(std::ostream& os, const ReportData& d) {
  const std::string equal_line(99, '=');
  const std::string dash_line(88, '-');
  const std::string dash_line_short(55, '-');
  const std::string dot_line(56, '.');
  const size_t prec = 20;
  const size_t ckw = prec + 8;
  size_t nw = 0;
  for (const KernelRow& k : d.kernels) {
    nw = std::max(nw, k.name.size());
    for (size_t v = 0; v < d.variants.size(); ++v)
      for (const std::string& t : d.tunings[v])
        nw = std::max(nw, d.variants[v].size() + 1 + t.size());
  }
  ++nw;
  os << equal_line << "\n" << "Checksum Report " << "\n" << equal_line << "\n";
  os << std::left << std::setw(nw) << "Kernel  " << "\n" << dot_line << "\n";
  os << std::left << std::setw(nw) << "Variants  " << std::left << std::setw(ckw)
     << "Checksum  " << std::left << std::setw(ckw) << "Checksum Diff  " << "\n";
  os << std::left << std::setw(nw) << "  " << std::left << std::setw(ckw) << "  "
     << std::left << std::setw(ckw) << "(vs. first variant listed)  " << "\n";
  os << dash_line << "\n";
  for (const KernelRow& k : d.kernels) {
    os << std::left << std::setw(nw) << k.name << "\n" << dot_line << "\n";
    // the first variant/tuning that ran is the reference for the differences
    long double ref = 0.0L;
    bool found = false;
    for (size_t v = 0; v < d.variants.size() && !found; ++v)
      for (size_t t = 0; t < k.cells[v].size() && !found; ++t)
        if (k.cells[v][t].run) {
          ref = k.cells[v][t].checksum;
          found = true;
        }
    for (size_t v = 0; v < d.variants.size(); ++v) {
      for (size_t t = 0; t < d.tunings[v].size(); ++t) {
        const Cell& cell = k.cells[v][t];
        if (!cell.defined) continue;  // the suite lists only the kernel's own tunings
        const std::string label = d.variants[v] + "-" + d.tunings[v][t];
        if (cell.run) {
          os << std::left << std::setw(nw) << label << std::showpoint << std::setprecision(prec)
             << std::left << std::setw(ckw) << cell.checksum << std::left << std::setw(ckw)
             << (ref - cell.checksum) << "\n";
          os << std::noshowpoint;
        } else {
          os << std::left << std::setw(nw) << label << std::left << std::setw(ckw) << "Not Run"
             << std::left << std::setw(ckw) << "Not Run" << "\n";
        }
      }
    }
    os << "\n" << dash_line_short << "\n";
  }
  os.flush();
}

namespace {

struct FOMGroup {
  std::vector<size_t> variants;
};

std::vector<FOMGroup> fomGroups(const ReportData& d) {
  std::vector<FOMGroup> groups;
  for (size_t v = 0; v < d.variants.size(); ++v) {
    const std::string& name = d.variants[v];
    if (name.find("Base") == std::string::npos) continue;
    FOMGroup g;
    g.variants.push_back(v);
    const std::string::size_type pos = name.find('_');
    const std::string pm = pos == std::string::npos ? name : name.substr(pos + 1);
    for (size_t w = v + 1; w < d.variants.size(); ++w)
      if (d.variants[w].find(pm) != std::string::npos) g.variants.push_back(w);
    groups.push_back(g);
  }
  return groups;
}

}  // namespace

bool hasFOMGroups(const ReportData& d) { return !fomGroups(d).empty(); }

void writeFOMReport(std::ostream& os, const ReportData& d) {
  const std::vector<FOMGroup> groups = fomGroups(d);
  if (groups.empty()) return;
  const size_t kw = kernelColumnWidth(d);
  const size_t prec = 2;
  size_t fw = prec + 14;
  std::vector<size_t> ncols(groups.size(), 0);
  for (size_t g = 0; g < groups.size(); ++g) {
    for (size_t v : groups[g].variants) {
      ncols[g] += d.tunings[v].size();
      for (const std::string& t : d.tunings[v])
        fw = std::max(fw, d.variants[v].size() + 1 + t.size());
    }
  }
  const std::string pass(",        "), fail(",OVER_TOL"), base(",base_ref");
  os << "FOM Report : signed speedup(-)/slowdown(+) for each PM (base vs. RAJA) -> "
        "(T_RAJA - T_base) / T_base )";
  for (size_t g = 0; g < groups.size(); ++g)
    for (size_t i = 0; i < ncols[g] * 2; ++i) os << kSep;
  os << "\n";
  os << "'OVER_TOL' in column to right if RAJA speedup is over tolerance";
  for (size_t g = 0; g < groups.size(); ++g)
    for (size_t i = 0; i < ncols[g] * 2; ++i) os << kSep;
  os << "\n";
  os << std::left << std::setw(kw) << kKernelHead;
  for (const FOMGroup& g : groups)
    for (size_t v : g.variants)
      for (const std::string& t : d.tunings[v])
        os << kSep << std::left << std::setw(fw) << (d.variants[v] + "-" + t) << pass;
  os << "\n";

  // per group and column: executions, min, max, sum, and the per-kernel values
  std::vector<std::vector<int>> count(groups.size());
  std::vector<std::vector<double>> cmin(groups.size()), cmax(groups.size()), cavg(groups.size()),
      cdev(groups.size());
  for (size_t g = 0; g < groups.size(); ++g) {
    count[g].assign(ncols[g], 0);
    cmin[g].assign(ncols[g], std::numeric_limits<double>::max());
    cmax[g].assign(ncols[g], -std::numeric_limits<double>::max());
    cavg[g].assign(ncols[g], 0.0);
    cdev[g].assign(ncols[g], 0.0);
  }
  std::vector<std::vector<std::vector<double>>> pct(
      d.kernels.size(), std::vector<std::vector<double>>(groups.size()));
  os << std::setprecision(prec);
  for (size_t ik = 0; ik < d.kernels.size(); ++ik) {
    const KernelRow& k = d.kernels[ik];
    os << std::left << std::setw(kw) << k.name;
    for (size_t g = 0; g < groups.size(); ++g) {
      pct[ik][g].assign(ncols[g], 0.0);
      double base_tot = -1.0;
      size_t col = 0;
      for (size_t v : groups[g].variants) {
        for (size_t t = 0; t < d.tunings[v].size(); ++t, ++col) {
          const Cell& cell = k.cells[v][t];
          if (cell.run) {
            ++count[g][col];
            const bool is_base = base_tot < 0.0;
            if (is_base) base_tot = cell.tot_time;
            const double p = base_tot > 0.0 ? (cell.tot_time - base_tot) / base_tot : 0.0;
            pct[ik][g][col] = p;
            const std::string& tag = is_base ? base : (p > d.pf_tolerance ? fail : pass);
            os << kSep << std::setw(fw) << std::left << p << std::right << tag;
            cmin[g][col] = std::min(cmin[g][col], p);
            cmax[g][col] = std::max(cmax[g][col], p);
            cavg[g][col] += p;
          } else {
            os << kSep << std::left << std::setw(fw) << 0.0 << pass;
          }
        }
      }
    }
    os << "\n";
  }
  for (size_t g = 0; g < groups.size(); ++g)
    for (size_t c = 0; c < ncols[g]; ++c) cavg[g][c] = count[g][c] > 0 ? cavg[g][c] / count[g][c] : 0.0;
  for (size_t ik = 0; ik < d.kernels.size(); ++ik) {
    for (size_t g = 0; g < groups.size(); ++g) {
      size_t col = 0;
      for (size_t v : groups[g].variants)
        for (size_t t = 0; t < d.tunings[v].size(); ++t, ++col)
          if (d.kernels[ik].cells[v][t].run) {
            const double e = pct[ik][g][col] - cavg[g][col];
            cdev[g][col] += e * e;
          }
    }
  }
  // the suite divides the squared deviations by the count and reports that
  // (Executor.cpp:1230-1240), without a square root
  for (size_t g = 0; g < groups.size(); ++g)
    for (size_t c = 0; c < ncols[g]; ++c) cdev[g][c] = count[g][c] > 0 ? cdev[g][c] / count[g][c] : 0.0;
  os << std::left << std::setw(kw) << " ";
  for (size_t g = 0; g < groups.size(); ++g)
    for (size_t c = 0; c < ncols[g]; ++c) os << kSep << std::setw(fw) << std::left << "  " << std::right << pass;
  os << "\n";
  const char* names[] = {"Col Min", "Col Max", "Col Avg", "Col Std Dev"};
  const std::vector<std::vector<double>>* rows[] = {&cmin, &cmax, &cavg, &cdev};
  for (int r = 0; r < 4; ++r) {
    os << std::left << std::setw(kw) << names[r];
    for (size_t g = 0; g < groups.size(); ++g)
      for (size_t c = 0; c < ncols[g]; ++c)
        os << kSep << std::left << std::setw(fw) << (*rows[r])[g][c] << pass;
    os << "\n";
  }
  os.flush();
}

void writeKernelInfo(std::ostream& os, const ReportData& d) {
  os << "Kernels run without MPI" << "\n";
  const std::string head("Kernels");
  size_t kw = head.size();
  long long mx[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (const KernelRow& k : d.kernels) {
    kw = std::max(kw, k.name.size());
    const long long v[9] = {k.problem_size, k.reps, k.its_per_rep, 0, k.bytes_per_rep,
                            k.flops_per_rep, k.bytes_read_per_rep, k.bytes_written_per_rep,
                            k.bytes_atomic_modify_written_per_rep};
    for (int i = 0; i < 9; ++i) mx[i] = std::max(mx[i], v[i]);
  }
  kw += 2;
  const char* heads[9] = {"Problem size", "Reps", "Iterations/rep", "Kernels/rep",
                          "Bytes/rep", "FLOPS/rep", "BytesRead/rep", "BytesWritten/rep",
                          "BytesAtomicModifyWritten/rep"};
  // a column is as wide as its heading or the digits of its largest value
  // (log10 of it, truncated), plus 3; Kernels/rep at least 4
  size_t w[9];
  for (int i = 0; i < 9; ++i) {
    const size_t hw = std::string(heads[i]).size();
    if (i == 3) {
      w[i] = std::max<size_t>(hw, 4);
    } else {
      const double lg = std::log10(static_cast<double>(mx[i]));
      const long long digits = std::isfinite(lg) ? static_cast<long long>(lg) : 0;
      w[i] = static_cast<size_t>(std::max<long long>(static_cast<long long>(hw), digits)) + 3;
    }
  }
  os << std::left << std::setw(kw) << head;
  for (int i = 0; i < 9; ++i) os << kSep << std::right << std::setw(w[i]) << heads[i];
  os << "\n";
  for (const KernelRow& k : d.kernels) {
    const long long v[9] = {k.problem_size, k.reps, k.its_per_rep, k.kernels_per_rep,
                            k.bytes_per_rep, k.flops_per_rep, k.bytes_read_per_rep,
                            k.bytes_written_per_rep, k.bytes_atomic_modify_written_per_rep};
    os << std::left << std::setw(kw) << k.name;
    for (int i = 0; i < 9; ++i) os << kSep << std::right << std::setw(w[i]) << v[i];
    os << "\n";
  }
  os.flush();
}

}  // namespace reports
}  // namespace rajaperf
