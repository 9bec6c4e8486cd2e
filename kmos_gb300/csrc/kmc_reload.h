// kmc_reload.h -- kmos .reload files (base.mpy:363-578, base_otf.f90:448-663; both
// backends write the same layout): gfortran-style number formatting, the reader, the
// writer, and the consistency check of the avail_sites columns a file holds.  Shared by
// the pool trajectories (kmc_state.cu) and the otf batches (kmc_otf.cu).
#pragma once

#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "kmc_host.h"

namespace kmc_reload {
using kmc_host::fail;

// ------------------------------------------------------------ Fortran-style output
// ESw.d edit descriptor as gfortran writes it: one digit before the point, d after,
// exponent "E+dd" (|e| < 100) or "+ddd" (|e| >= 100), right-justified in w columns,
// w asterisks when it does not fit.
inline std::string fmt_es(double v, int w, int d) {
  std::string s;
  if (std::isnan(v)) {
    s = "NaN";
  } else if (std::isinf(v)) {
    s = v < 0 ? "-Infinity" : "Infinity";
    if ((int)s.size() > w) s = v < 0 ? "-Inf" : "Inf";
  } else {
    char tmp[64];
    snprintf(tmp, sizeof(tmp), "%.*E", d, v);
    s = tmp;
    const size_t e = s.find('E');
    const int ex = atoi(s.c_str() + e + 1);
    if (ex <= -100 || ex >= 100) s = s.substr(0, e) + s.substr(e + 1);  // "1.23+100"
  }
  if ((int)s.size() > w) return std::string(w, '*');
  return std::string(w - s.size(), ' ') + s;
}

inline std::string fmt_i(int64_t v, int w) {
  char tmp[32];
  snprintf(tmp, sizeof(tmp), "%lld", (long long)v);
  std::string s = tmp;
  if ((int)s.size() > w) return std::string(w, '*');
  return std::string(w - s.size(), ' ') + s;
}

inline std::string fmt_exact(double v) {
  char tmp[40];
  snprintf(tmp, sizeof(tmp), "%.17g", v);
  return tmp;
}

// Number token as a Fortran list-directed read takes it: also "1.5+100" and "1.5D+03".
inline bool parse_real(const std::string &tok, double *out) {
  std::string t = tok;
  for (auto &c : t)
    if (c == 'D' || c == 'd') c = 'E';
  if (t.find_first_of("eE") == std::string::npos) {
    const size_t k = t.find_first_of("+-", 1);
    if (k != std::string::npos && (isdigit((unsigned char)t[k - 1]) || t[k - 1] == '.')) t.insert(k, "E");
  }
  errno = 0;
  char *end = nullptr;
  const double v = strtod(t.c_str(), &end);
  if (end == t.c_str() || *end != 0) return false;
  *out = v;
  return true;
}

inline bool parse_int(const std::string &tok, int64_t *out) {
  errno = 0;
  char *end = nullptr;
  const long long v = strtoll(tok.c_str(), &end, 10);
  if (end == tok.c_str() || *end != 0 || errno) return false;
  *out = v;
  return true;
}

inline std::vector<std::string> split(const std::string &line) {
  std::vector<std::string> out;
  size_t i = 0;
  while (i < line.size()) {
    while (i < line.size() && (line[i] == ' ' || line[i] == '\t' || line[i] == '\r' || line[i] == ',')) i++;
    const size_t j = i;
    while (i < line.size() && !(line[i] == ' ' || line[i] == '\t' || line[i] == '\r' || line[i] == ',')) i++;
    if (i > j) out.push_back(line.substr(j, i - j));
  }
  return out;
}

inline bool read_line(FILE *f, std::string &line) {
  line.clear();
  char buf[65536];
  bool any = false;
  while (fgets(buf, sizeof(buf), f)) {
    any = true;
    line += buf;
    if (!line.empty() && line.back() == '\n') {
      line.pop_back();
      return true;
    }
  }
  return any;
}

// Contents of a .reload file.
struct ReloadFile {
  bool have_proc = false, have_volume = false, have_time = false, have_step = false, have_lattice = false;
  bool have_nsites = false, have_rates = false, have_procstat = false, have_walltime = false;
  int64_t nr_of_proc = 0, volume = 0, kmc_step = 0;
  double kmc_time = 0.0, walltime = 0.0;
  std::vector<int64_t> lattice, nsites, procstat;
  std::vector<double> rates;
  std::vector<std::vector<int64_t>> as1, as2;
  // "#gb300" lines
  int32_t dims[3] = {0, 0, 0};
  bool exact_time = false, exact_rates = false, exact_integ = false, have_dt = false, have_rng = false;
  double x_kmc_time = 0.0, x_dt = 0.0;
  std::vector<double> x_rates, x_integ;
  int32_t rng_kind = 0;
  uint32_t seed = 0, traj = 0;
  uint64_t rng[4] = {0, 0, 0, 0};
};

inline int parse_reload(const char *path, ReloadFile &r, bool header_only) {
  FILE *f = fopen(path, "r");
  if (!f) return fail(KMC_ERR_ARG, std::string("cannot open ") + path);
  std::string line;
  int rc = KMC_OK;
  auto bad = [&](const std::string &what) { rc = fail(KMC_ERR_ARG, std::string(path) + ": bad " + what); };
  auto ints = [&](const std::vector<std::string> &tok, size_t from, std::vector<int64_t> &out) {
    out.clear();
    for (size_t i = from; i < tok.size(); i++) {
      int64_t v;
      if (!parse_int(tok[i], &v)) return false;
      out.push_back(v);
    }
    return true;
  };
  auto reals = [&](const std::vector<std::string> &tok, size_t from, std::vector<double> &out) {
    out.clear();
    for (size_t i = from; i < tok.size(); i++) {
      double v;
      if (!parse_real(tok[i], &v)) return false;
      out.push_back(v);
    }
    return true;
  };
  while (rc == KMC_OK && read_line(f, line)) {
    const std::vector<std::string> tok = split(line);
    if (tok.empty()) continue;
    if (tok[0][0] == '#') {
      if (tok[0] != "#gb300" || tok.size() < 2) continue;
      const std::string &k = tok[1];
      if (k == "system_size" && tok.size() == 5) {
        for (int i = 0; i < 3; i++) {
          int64_t v;
          if (!parse_int(tok[2 + i], &v) || v < 1 || v > (1 << 28)) { bad("#gb300 system_size"); break; }
          r.dims[i] = (int32_t)v;
        }
      }
      if (header_only) continue;
      if (k == "kmc_time" && tok.size() == 3) r.exact_time = parse_real(tok[2], &r.x_kmc_time);
      else if (k == "kmc_time_step" && tok.size() == 3) r.have_dt = parse_real(tok[2], &r.x_dt);
      else if (k == "rates") r.exact_rates = reals(tok, 2, r.x_rates);
      else if (k == "integ_rates") r.exact_integ = reals(tok, 2, r.x_integ);
      else if (k == "rng") {
        // kind, seed, trajectory id, four state words; a line that is there but does not
        // read is refused rather than skipped (the trajectory would keep another stream)
        int64_t kind, seed, traj;
        bool ok = tok.size() == 9 && parse_int(tok[2], &kind) && parse_int(tok[3], &seed) &&
                  parse_int(tok[4], &traj) && seed >= 0 && seed <= 0xFFFFFFFFll && traj >= 0 &&
                  traj <= 0xFFFFFFFFll;
        for (int i = 0; i < 4 && ok; i++) {
          errno = 0;
          char *end = nullptr;
          r.rng[i] = strtoull(tok[5 + i].c_str(), &end, 10);
          ok = end != tok[5 + i].c_str() && *end == 0 && !errno && tok[5 + i][0] != '-';
        }
        if (!ok) { bad("#gb300 rng"); break; }
        r.have_rng = true;
        r.rng_kind = kind >= 0 && kind <= 1 ? (int32_t)kind : -1;  // -1: refused by read_reload
        r.seed = (uint32_t)seed;
        r.traj = (uint32_t)traj;
      }
      continue;
    }
    const std::string &label = tok[0];
    int64_t v;
    if (label == "nr_of_proc") {
      if (tok.size() != 2 || !parse_int(tok[1], &v)) bad("nr_of_proc"); else { r.nr_of_proc = v; r.have_proc = true; }
    } else if (label == "volume") {
      if (tok.size() != 2 || !parse_int(tok[1], &v)) bad("volume"); else { r.volume = v; r.have_volume = true; }
    } else if (header_only) {
      continue;
    } else if (label == "kmc_time") {
      if (tok.size() != 2 || !parse_real(tok[1], &r.kmc_time)) bad("kmc_time"); else r.have_time = true;
    } else if (label == "walltime") {
      if (tok.size() == 2 && parse_real(tok[1], &r.walltime)) r.have_walltime = true;
    } else if (label == "kmc_step") {
      if (tok.size() != 2 || !parse_int(tok[1], &r.kmc_step)) bad("kmc_step"); else r.have_step = true;
    } else if (label == "lattice") {
      if (!ints(tok, 1, r.lattice)) bad("lattice"); else r.have_lattice = true;
    } else if (label == "nr_of_sites") {
      if (!ints(tok, 1, r.nsites)) bad("nr_of_sites"); else r.have_nsites = true;
    } else if (label == "rates") {
      if (!reals(tok, 1, r.rates)) bad("rates"); else r.have_rates = true;
    } else if (label == "procstat") {
      if (!ints(tok, 1, r.procstat)) bad("procstat"); else r.have_procstat = true;
    } else if (label == "avail_sites" || label == "avail_sites_back") {
      std::vector<int64_t> row;
      if (tok.size() < 2 || !parse_int(tok[1], &v) || v < 1 || v > 256 || !ints(tok, 2, row)) { bad(label); break; }
      auto &dst = label == "avail_sites" ? r.as1 : r.as2;
      if ((int64_t)dst.size() < v) dst.resize(v);
      dst[v - 1] = std::move(row);
    }
  }
  fclose(f);
  return rc;
}


// What save_system writes (base.mpy:528-575, edit descriptor by edit descriptor), plus
// the "#gb300" lines.  as1[q] holds the nsites[q] entries of avail_sites(q+1, :, 1).
struct ReloadData {
  int P = 0, V = 0;
  int32_t dims[3] = {0, 0, 0};
  double kmc_time = 0.0, kmc_time_step = 0.0, walltime = 0.0;
  int64_t kmc_step = 0;
  int32_t rng_kind = 0;
  uint32_t seed = 0, traj = 0;
  uint64_t rng[4] = {0, 0, 0, 0};
  std::vector<double> rates, integ;
  std::vector<int64_t> procstat;
  std::vector<int32_t> nsites, lattice;
  std::vector<std::vector<int32_t>> as1;
};

inline int write_reload(const char *path, const ReloadData &d) {
  const int P = d.P, V = d.V;
  FILE *f = fopen(path, "w");
  if (!f) return fail(KMC_ERR_ARG, std::string("cannot write ") + path);
  std::string s;
  s.reserve(64 + (size_t)V * 9 * (2 * P + 1));
  s += "#Reload file written by kmos. Do not edit manually!\n";
  s += "#Scalar variables\n";
  s += " kmc_time  " + fmt_es(d.kmc_time, 22, 15) + "\n";
  s += " walltime   " + fmt_es(d.walltime, 13, 7) + "\n";
  s += " kmc_step " + fmt_i(d.kmc_step, 22) + "\n";
  s += " nr_of_proc " + fmt_i(P, 12) + "\n";     // list-directed: default integer, 12 columns
  s += " volume " + fmt_i(V, 12) + "\n";
  // what the reference's file cannot hold exactly; its reader skips comment lines
  s += "#gb300 system_size " + std::to_string(d.dims[0]) + " " + std::to_string(d.dims[1]) + " " +
       std::to_string(d.dims[2]) + "\n";
  s += "#gb300 kmc_time " + fmt_exact(d.kmc_time) + "\n";
  s += "#gb300 kmc_time_step " + fmt_exact(d.kmc_time_step) + "\n";
  s += "#gb300 rng " + std::to_string(d.rng_kind) + " " + std::to_string(d.seed) + " " + std::to_string(d.traj);
  for (int i = 0; i < 4; i++) s += " " + std::to_string((unsigned long long)d.rng[i]);
  s += "\n#gb300 rates";
  for (int i = 0; i < P; i++) s += " " + fmt_exact(d.rates[i]);
  s += "\n#gb300 integ_rates";
  for (int i = 0; i < P; i++) s += " " + fmt_exact(d.integ[i]);
  s += "\n#Vector variables\n";
  s += "procstat ";
  for (int i = 0; i < P; i++) s += fmt_i(d.procstat[i], 21);
  s += "\nnr_of_sites ";
  for (int i = 0; i < P; i++) s += fmt_i(d.nsites[i], 9);
  s += "\nrates ";
  for (int i = 0; i < P; i++) s += fmt_es(d.rates[i], 14, 7);
  s += "\nlattice ";
  for (int i = 0; i < V; i++) s += fmt_i(d.lattice[i], 9);
  s += "\n";
  std::vector<int32_t> row(V + 1);
  for (int q = 0; q < P; q++) {
    s += "avail_sites " + fmt_i(q + 1, 9);
    for (int i = 1; i <= V; i++) s += fmt_i(i <= d.nsites[q] ? d.as1[q][i - 1] : 0, 9);
    s += "\n";
  }
  for (int q = 0; q < P; q++) {
    std::fill(row.begin(), row.end(), 0);
    for (int i = 1; i <= d.nsites[q]; i++) row[d.as1[q][i - 1]] = i;
    s += "avail_sites_back " + fmt_i(q + 1, 9);
    for (int i = 1; i <= V; i++) s += fmt_i(row[i], 9);
    s += "\n";
  }
  const bool ok = fwrite(s.data(), 1, s.size(), f) == s.size();
  if (fclose(f) != 0 || !ok) return fail(KMC_ERR_ARG, std::string("short write to ") + path);
  return KMC_OK;
}

// The second pass of reload_system into a model of P processes on V sites: every vector
// present with its length, species in -1..nspecies, and each process's two avail_sites
// columns inverse to each other over its first nr_of_sites entries (zero past them), a
// "#gb300 rng" line of a known stream.  Fills d's vectors (as1 entries per process; rates and integ_rates exact where the
// file's "#gb300" lines hold them, integ_rates 0 otherwise) and scalars.
inline int read_reload(const ReloadFile &r, int P, int V, int nspecies, ReloadData &d) {
  if (!r.have_proc || r.nr_of_proc != P) return fail(KMC_ERR_ARG, "reload file: nr_of_proc differs from the model");
  if (!r.have_volume || r.volume != V) return fail(KMC_ERR_ARG, "reload file: volume differs from the system");
  if (!r.have_time || !r.have_step || !r.have_lattice || !r.have_nsites || !r.have_rates || !r.have_procstat)
    return fail(KMC_ERR_ARG, "reload file lacks one of kmc_time, kmc_step, lattice, nr_of_sites, rates, procstat");
  if ((int)r.lattice.size() != V || (int)r.nsites.size() != P || (int)r.rates.size() != P ||
      (int)r.procstat.size() != P || (int)r.as1.size() != P || (int)r.as2.size() != P)
    return fail(KMC_ERR_ARG, "reload file: a vector has the wrong length");
  d.P = P;
  d.V = V;
  d.lattice.resize(V);
  for (int i = 0; i < V; i++) {
    if (r.lattice[i] < -1 || r.lattice[i] > nspecies) return fail(KMC_ERR_ARG, "reload file: unknown species");
    d.lattice[i] = (int32_t)r.lattice[i];
  }
  d.as1.assign(P, {});
  d.nsites.assign(P, 0);
  d.procstat.assign(P, 0);
  d.rates.assign(P, 0.0);
  d.integ.assign(P, 0.0);
  for (int q = 0; q < P; q++) {
    const auto &a1 = r.as1[q], &a2 = r.as2[q];
    if ((int)a1.size() != V || (int)a2.size() != V) return fail(KMC_ERR_ARG, "reload file: avail_sites row length");
    const int64_t n = r.nsites[q];
    if (n < 0 || n > V) return fail(KMC_ERR_TABLE, "reload file: nr_of_sites out of range");
    int64_t back = 0;
    for (int i = 0; i < V; i++) {
      const int64_t s = a1[i];
      if (i < n) {
        if (s < 1 || s > V || a2[s - 1] != i + 1) return fail(KMC_ERR_TABLE, "reload file: avail_sites columns disagree");
        d.as1[q].push_back((int32_t)s);
      } else if (s != 0) {
        return fail(KMC_ERR_TABLE, "reload file: avail_sites entry past nr_of_sites");
      }
      if (a2[i] != 0) back++;
    }
    if (back != n) return fail(KMC_ERR_TABLE, "reload file: avail_sites_back has extra entries");
    d.nsites[q] = (int32_t)n;
    d.procstat[q] = r.procstat[q];
    d.rates[q] = r.exact_rates && (int)r.x_rates.size() == P ? r.x_rates[q] : r.rates[q];
    d.integ[q] = r.exact_integ && (int)r.x_integ.size() == P ? r.x_integ[q] : 0.0;
  }
  d.kmc_time = r.exact_time ? r.x_kmc_time : r.kmc_time;
  d.kmc_step = r.kmc_step;
  d.kmc_time_step = r.have_dt ? r.x_dt : 0.0;
  d.walltime = r.have_walltime ? r.walltime : 0.0;
  for (int i = 0; i < 3; i++) d.dims[i] = r.dims[i];
  if (r.have_rng) {
    // the "#gb300 rng" line: a known stream, and for the gfortran one a xoshiro256**
    // state that is not all zero (that state only ever yields zero)
    if (r.rng_kind != kmc::RNG_GFORTRAN && r.rng_kind != kmc::RNG_PHILOX)
      return fail(KMC_ERR_ARG, "reload file: unknown random stream");
    if (r.rng_kind == kmc::RNG_GFORTRAN && !(r.rng[0] | r.rng[1] | r.rng[2] | r.rng[3]))
      return fail(KMC_ERR_ARG, "reload file: all-zero gfortran random state");
    d.rng_kind = r.rng_kind;
    d.seed = r.seed;
    d.traj = r.traj;
    for (int i = 0; i < 4; i++) d.rng[i] = r.rng[i];
  }
  return KMC_OK;
}

}  // namespace kmc_reload
