// Autotuner: picks the FFT radix plans, line splits, stage-kernel row layouts
// and subspace-kernel shapes of a handle by timing the candidates on the
// handle's own tables and buffers, and keeps the choices in a JSON cache.
//
// What it chooses (every candidate computes the same result; only the
// rounding of the transforms differs):
//   fft    the radix sequence of each grid-FFT length (Stockham stages of
//          radix 2, 3, 4, 5, 7, 8, 11, 13 in any order: Hartree, Kerker and
//          fft3d transforms), timed on a forward + backward full-grid pass;
//   lines  register / fixed-length line kernels against the shared-memory
//          four-step kernels with a runtime split n = a * b (a, b <= 16) per
//          length, timed on a full H.psi;
//   rows   the row layout each grid-size class's H.psi stage kernels are
//          dispatched with (the tightest layout holding the class's spheres,
//          the compact N/4 + 1 rows, or every row), timed on a full H.psi;
//   chunk  the items per chunk of the three H.psi stage launches (all, or
//          2048 ... 128: a chunk whose x-plane buffer fits in L2 reads it back
//          from L2), timed on a full H.psi;
//   overlap tensor cores or CUDA cores and the split-K length (512 ... 8192
//          coefficients per CTA) of S = X^H X (tensor cores only for
//          subspaces of 64 bands or more: accuracy, see kTcMinBands);
//   rotate tensor cores or CUDA cores for X <- X C (the same rule);
//   jacobi one CTA per k-set or a two-CTA cluster.
// The reference plans its FFTs with FFTW_ESTIMATE (Source/fft.f90:204-212),
// which picks a plan by heuristics without timing; it has no GPU kernels.
//
// The cache file is a JSON object keyed by device (name and SM count), each
// holding "key": "value" strings; keys name the shape a choice was timed on.
// Tuning overwrites the handle's wavefunction buffers, the H psi buffer and
// the subspace matrices (an SCF starts from its own start vectors), so call it
// right after derek_gpu_create.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <set>
#include <sstream>
#include <string>
#include <vector>

#include "handle.h"
#include "scf_kernels.cuh"

using namespace derek;

namespace {

using Cache = std::map<std::string, std::map<std::string, std::string>>;

// ---- a small reader and writer for the cache's two-level JSON object -------
struct JsonIn {
  const std::string &s;
  size_t i = 0;
  explicit JsonIn(const std::string &t) : s(t) {}
  void ws() {
    while (i < s.size() && (s[i] == ' ' || s[i] == '\n' || s[i] == '\r' || s[i] == '\t')) ++i;
  }
  bool eat(char c) {
    ws();
    if (i < s.size() && s[i] == c) {
      ++i;
      return true;
    }
    return false;
  }
  bool str(std::string &out) {
    ws();
    if (i >= s.size() || s[i] != '"') return false;
    ++i;
    out.clear();
    while (i < s.size() && s[i] != '"') {
      if (s[i] == '\\' && i + 1 < s.size()) ++i;
      out.push_back(s[i++]);
    }
    if (i >= s.size()) return false;
    ++i;
    return true;
  }
};

bool parse_cache(const std::string &text, Cache &out) {
  JsonIn in(text);
  if (!in.eat('{')) return false;
  if (in.eat('}')) return true;
  do {
    std::string dev;
    if (!in.str(dev) || !in.eat(':') || !in.eat('{')) return false;
    auto &m = out[dev];
    if (!in.eat('}')) {
      do {
        std::string k, v;
        if (!in.str(k) || !in.eat(':') || !in.str(v)) return false;
        m[k] = v;
      } while (in.eat(','));
      if (!in.eat('}')) return false;
    }
  } while (in.eat(','));
  return in.eat('}');
}

std::string quote(const std::string &x) {
  std::string o = "\"";
  for (char c : x) {
    if (c == '"' || c == '\\') o.push_back('\\');
    o.push_back(c);
  }
  return o + "\"";
}

std::string write_cache(const Cache &c) {
  std::ostringstream o;
  o << "{\n";
  size_t d = 0;
  for (const auto &dev : c) {
    o << " " << quote(dev.first) << ": {\n";
    size_t j = 0;
    for (const auto &kv : dev.second)
      o << "  " << quote(kv.first) << ": " << quote(kv.second) << (++j < dev.second.size() ? ",\n" : "\n");
    o << " }" << (++d < c.size() ? ",\n" : "\n");
  }
  o << "}\n";
  return o.str();
}

// ---- candidates -------------------------------------------------------------
std::string radix_str(const FftPlan &p) {
  std::string s;
  for (int i = 0; i < p.nstages; ++i) s += (i ? "x" : "") + std::to_string(p.radix[i]);
  return s;
}

bool parse_radices(const std::string &s, int n, FftPlan &p) {
  int r[kMaxRadices], ns = 0, prod = 1;
  std::istringstream in(s);
  std::string tok;
  while (std::getline(in, tok, 'x')) {
    if (ns >= kMaxRadices) return false;
    const int v = std::atoi(tok.c_str());
    if (v != 2 && v != 3 && v != 4 && v != 5 && v != 7 && v != 8 && v != 11 && v != 13) return false;
    r[ns++] = v;
    prod *= v;
  }
  if (prod != n || ns == 0) return false;
  p.nstages = ns;
  for (int i = 0; i < ns; ++i) p.radix[i] = r[i];
  return true;
}

// radix sequences for n: the power of two as 8s, 4s and 2s in a few
// groupings, the odd primes as themselves, in several orders
std::vector<std::string> radix_candidates(int n) {
  int m = n, e2 = 0;
  while (m % 2 == 0) m /= 2, ++e2;
  std::vector<int> odd;
  for (int p : {3, 5, 7, 11, 13})
    while (m % p == 0) m /= p, odd.push_back(p);
  if (m != 1) return {};
  std::vector<std::vector<int>> pow2s;
  auto group = [&](int big) {
    std::vector<int> g;
    int e = e2;
    while (e >= 3 && big >= 8) g.push_back(8), e -= 3;
    while (e >= 2) g.push_back(4), e -= 2;
    while (e >= 1) g.push_back(2), e -= 1;
    return g;
  };
  pow2s.push_back(group(8));
  pow2s.push_back(group(4));
  if (e2 >= 1) pow2s.push_back(std::vector<int>(e2, 2));
  std::set<std::string> seen;
  std::vector<std::string> out;
  for (const auto &p2 : pow2s) {
    std::vector<int> desc = p2, asc = p2, od = odd, odr = odd;
    std::sort(desc.rbegin(), desc.rend());
    std::sort(asc.begin(), asc.end());
    std::sort(odr.rbegin(), odr.rend());
    std::vector<std::vector<int>> orders;
    std::vector<int> a = desc;
    a.insert(a.end(), od.begin(), od.end());
    orders.push_back(a);
    std::vector<int> b = od;
    b.insert(b.end(), desc.begin(), desc.end());
    orders.push_back(b);
    std::vector<int> c = asc;
    c.insert(c.end(), odr.begin(), odr.end());
    orders.push_back(c);
    std::vector<int> d = odr;
    d.insert(d.end(), asc.begin(), asc.end());
    orders.push_back(d);
    for (const auto &o : orders) {
      if (o.empty() || (int)o.size() > kMaxRadices) continue;
      std::string s;
      for (size_t i = 0; i < o.size(); ++i) s += (i ? "x" : "") + std::to_string(o[i]);
      if (seen.insert(s).second) out.push_back(s);
    }
  }
  return out;
}

std::vector<std::pair<int, int>> split_candidates(int n) {
  std::vector<std::pair<int, int>> out;
  for (int a = 1; a <= 16; ++a)
    if (n % a == 0 && n / a <= 16) out.push_back({a, n / a});
  return out;
}

// ---- timing -------------------------------------------------------------------
struct Timer {
  cudaEvent_t a = nullptr, b = nullptr;
  Timer() {
    cudaEventCreate(&a);
    cudaEventCreate(&b);
  }
  ~Timer() {
    cudaEventDestroy(a);
    cudaEventDestroy(b);
  }
  // best of `reps` timed runs after one warm-up run (ms)
  template <typename F> float best(derek_gpu *h, int reps, F &&f) {
    f();
    float best = 1e30f;
    for (int r = 0; r < reps; ++r) {
      cudaEventRecord(a, h->stream);
      f();
      cudaEventRecord(b, h->stream);
      cudaEventSynchronize(b);
      float ms = 0;
      cudaEventElapsedTime(&ms, a, b);
      best = std::min(best, ms);
    }
    return best;
  }
};

const char *prec_name(const derek_gpu *h) { return h->prec == DEREK_PREC_FP64 ? "fp64" : "mixed"; }

std::string device_key() {
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceProp p{};
  cudaGetDeviceProperties(&p, dev);
  return std::string(p.name) + " (" + std::to_string(p.multiProcessorCount) + " SMs)";
}

int upload_sys(derek_gpu *h) {
  DEREK_CUDA(h, cudaMemcpyAsync(h->d_sys, h->sys.data(), h->sys.size() * sizeof(SysDev),
                                cudaMemcpyHostToDevice, h->stream));
  return DEREK_OK;
}

void set_radices(derek_gpu *h, int n, const FftPlan &p) {
  for (auto &S : h->sys)
    for (int i = 0; i < 3; ++i)
      if (S.plan[i].n == n) {
        S.plan[i].nstages = p.nstages;
        std::copy(p.radix, p.radix + kMaxRadices, S.plan[i].radix);
      }
}

void set_split(derek_gpu *h, int n, int a, int b) {
  for (auto &S : h->sys)
    for (int i = 0; i < 3; ++i)
      if (S.lp[i].n == n) {
        S.lp[i].a = a;
        S.lp[i].b = b;
        S.lp[i].group = 32 / std::max(a, b);
      }
}

std::vector<int> lengths(const derek_gpu *h) {
  std::set<int> s;
  for (const auto &S : h->sys)
    for (int i = 0; i < 3; ++i) s.insert(S.n[i]);
  return std::vector<int>(s.begin(), s.end());
}

int row_bound_for(int n, int variant, int max_m) {
  // 0: as tight as the class allows, 1: the compact N/4 + 1 rows, 2: every row
  if (variant == 0) return max_m;
  if (variant == 1) return std::max(max_m, n / 4 + 1);
  return std::max(max_m, n / 2);
}

const char *kRowNames[3] = {"tight", "compact", "all"};

struct Tuner {
  derek_gpu *h;
  std::map<std::string, std::string> &cache;   // this device's entries
  bool use_cache;
  Timer tm;
  int tuned = 0, cached = 0;

  bool lookup(const std::string &k, std::string &v) {
    if (!use_cache) return false;
    auto it = cache.find(k);
    if (it == cache.end()) return false;
    v = it->second;
    return true;
  }

  float time_hpsi() {
    return tm.best(h, 3, [&] { apply_h_items(h, 0, h->nitems, h->d_X, nullptr, h->d_HX, nullptr); });
  }

  int fft_radices() {
    for (int n : lengths(h)) {
      const std::string key = "fft n=" + std::to_string(n);
      std::string v;
      FftPlan p{};
      p.n = n;
      if (lookup(key, v) && parse_radices(v, n, p)) {
        set_radices(h, n, p);
        ++cached;
        continue;
      }
      float best = 1e30f;
      std::string best_s;
      for (const auto &cand : radix_candidates(n)) {
        if (!parse_radices(cand, n, p)) continue;
        set_radices(h, n, p);
        if (int st = upload_sys(h)) return st;
        const float ms = tm.best(h, 3, [&] {
          launch_fft3d_grid(h->tab, 0, h->nsys, h->max_nmax, h->d_cgrid, -1, h->stream);
          launch_fft3d_grid(h->tab, 0, h->nsys, h->max_nmax, h->d_cgrid, +1, h->stream);
        });
        if (ms < best) best = ms, best_s = cand;
      }
      if (best_s.empty()) continue;
      parse_radices(best_s, n, p);
      set_radices(h, n, p);
      cache[key] = best_s;
      ++tuned;
    }
    return upload_sys(h);
  }

  int lines() {
    const auto ns = lengths(h);
    std::string key = std::string("lines prec=") + prec_name(h) + " n=";
    for (size_t i = 0; i < ns.size(); ++i) key += (i ? "," : "") + std::to_string(ns[i]);
    std::string v;
    if (lookup(key, v)) {
      // "fixed" or "split 72:8x9 48:6x8"
      if (v == "fixed") {
        h->tune.generic_lines = 0;
        ++cached;
        return DEREK_OK;
      }
      if (v.rfind("split", 0) == 0) {
        std::istringstream in(v.substr(5));
        std::string tok;
        while (in >> tok) {
          int n = 0, a = 0, b = 0;
          if (std::sscanf(tok.c_str(), "%d:%dx%d", &n, &a, &b) == 3 && a * b == n && a <= 16 && b <= 16)
            set_split(h, n, a, b);
        }
        h->tune.generic_lines = 1;
        ++cached;
        return upload_sys(h);
      }
    }
    h->tune.generic_lines = 0;
    const float t_fixed = time_hpsi();
    h->tune.generic_lines = 1;
    float t_gen = time_hpsi();
    std::string splits;
    if (t_gen < 1.5f * t_fixed) {
      // search the splits of each length in turn (others at their current split)
      for (int n : ns) {
        int ba = 0, bb = 0;
        float best = 1e30f;
        for (auto ab : split_candidates(n)) {
          set_split(h, n, ab.first, ab.second);
          if (int st = upload_sys(h)) return st;
          const float ms = time_hpsi();
          if (ms < best) best = ms, ba = ab.first, bb = ab.second;
        }
        set_split(h, n, ba, bb);
        if (int st = upload_sys(h)) return st;
        t_gen = std::min(t_gen, best);
      }
    }
    for (int n : ns) {
      for (const auto &S : h->sys)
        for (int i = 0; i < 3; ++i)
          if (S.lp[i].n == n) {
            splits += " " + std::to_string(n) + ":" + std::to_string(S.lp[i].a) + "x" + std::to_string(S.lp[i].b);
            goto next;
          }
    next:;
    }
    h->tune.generic_lines = t_gen < t_fixed ? 1 : 0;
    cache[key] = h->tune.generic_lines ? "split" + splits : "fixed";
    ++tuned;
    return DEREK_OK;
  }

  int rows() {
    for (auto &c : h->classes) {
      const int n = c.n[0];
      if (c.n[1] != n || c.n[2] != n) continue;   // the register kernels serve cubic grids
      const std::string key = std::string("rows prec=") + prec_name(h) + " n=" + std::to_string(n) +
                              " m=" + std::to_string(c.max_m) + (h->tune.generic_lines ? " generic" : "");
      std::string v;
      if (lookup(key, v)) {
        for (int var = 0; var < 3; ++var)
          if (v == kRowNames[var]) c.disp_m = row_bound_for(n, var, c.max_m);
        ++cached;
        continue;
      }
      float best = 1e30f;
      int best_var = 0, last_bound = -1;
      for (int var = 0; var < 3; ++var) {
        const int bound = row_bound_for(n, var, c.max_m);
        if (bound == last_bound) continue;
        last_bound = bound;
        c.disp_m = bound;
        const float ms = time_hpsi();
        if (ms < best) best = ms, best_var = var;
      }
      c.disp_m = row_bound_for(n, best_var, c.max_m);
      cache[key] = kRowNames[best_var];
      ++tuned;
    }
    return DEREK_OK;
  }

  // items per chunk of the H.psi stage launches: the x-plane buffer of a
  // chunk that fits in L2 is re-read from L2 instead of HBM
  int chunks() {
    std::string key = std::string("hpsi_chunk prec=") + prec_name(h) + " items=" + std::to_string(h->nitems);
    for (const auto &c : h->classes) key += " " + std::to_string(c.n[0]) + ":" + std::to_string(c.count);
    std::string v;
    if (lookup(key, v)) {
      h->tune.hpsi_chunk = std::max(0, std::atoi(v.c_str()));
      ++cached;
      return DEREK_OK;
    }
    float best = 1e30f;
    int best_c = 0;
    for (int c : {0, 2048, 1024, 512, 256, 128}) {
      if (c >= h->nitems) continue;
      h->tune.hpsi_chunk = c;
      const float ms = time_hpsi();
      if (ms < best) best = ms, best_c = c;
    }
    h->tune.hpsi_chunk = best_c;
    cache[key] = std::to_string(best_c);
    ++tuned;
    return DEREK_OK;
  }

  std::string shape_key(const char *what) {
    return std::string(what) + " prec=" + prec_name(h) + " nb=" + std::to_string(h->max_nb_band) +
           " npw=" + std::to_string(h->max_npw_band) + " nks=" + std::to_string(h->nks);
  }

  // Tensor cores for the subspace products only where the subspace has at
  // least kTcMinBands carried bands (handle.h: the split-BF16 accuracy)
  bool tc_allowed() const { return tc_capable(h) && h->max_nb_band >= kTcMinBands; }

  int overlap() {
    const std::string key = shape_key("overlap");
    std::string v;
    if (lookup(key, v)) {
      char path[16] = {0};
      int ks = 0;
      if (std::sscanf(v.c_str(), "%15s %d", path, &ks) == 2 && ks >= kOverlapSplitMin && ks % kOverlapSplitMin == 0 &&
          (std::strcmp(path, "cuda") == 0 || tc_allowed())) {
        h->tune.overlap_tc = std::strcmp(path, "tc") == 0 ? 1 : 0;
        h->tune.ksplit = ks;
        ++cached;
        return DEREK_OK;
      }
    }
    float best = 1e30f;
    int best_tc = 0, best_ks = kOverlapSplit;
    for (int tc = 0; tc <= (tc_allowed() ? 1 : 0); ++tc)
      for (int ks : {kOverlapSplitMin, 2 * kOverlapSplitMin, kOverlapSplit, 2 * kOverlapSplit, 4 * kOverlapSplit}) {
        h->tune.overlap_tc = tc;
        h->tune.ksplit = ks;
        const float ms = tm.best(h, 3, [&] { overlap_all(h, h->d_X, h->d_X, h->d_S, 1); });
        if (ms < best) best = ms, best_tc = tc, best_ks = ks;
      }
    h->tune.overlap_tc = best_tc;
    h->tune.ksplit = best_ks;
    cache[key] = std::string(best_tc ? "tc " : "cuda ") + std::to_string(best_ks);
    ++tuned;
    return DEREK_OK;
  }

  int rotate() {
    if (!(tc_capable(h) && h->opts.use_tensor_cores != 1)) return DEREK_OK;
    const std::string key = shape_key("rotate");
    if (!tc_allowed()) {   // a rule, not a timing: nothing to cache
      h->tune.rotate_tc = 0;
      return DEREK_OK;
    }
    std::string v;
    if (lookup(key, v) && (v == "tc" || v == "cuda")) {
      h->tune.rotate_tc = v == "tc" ? 1 : 0;
      ++cached;
      return DEREK_OK;
    }
    // C = 0: the timed rotations zero the buffer, whose values do not matter here
    DEREK_CUDA(h, cudaMemsetAsync(h->d_C, 0, h->mat_off.empty() ? 0 :
               (size_t)(h->mat_off.back() + (long long)h->ks.back().nb * h->ks.back().nb) * sizeof(double2),
               h->stream));
    float best = 1e30f;
    int best_tc = 1;
    for (int tc = 1; tc >= 0; --tc) {
      h->tune.rotate_tc = tc;
      const float ms = tm.best(h, 3, [&] { rotate_all(h, h->d_Y, h->d_C); });
      if (ms < best) best = ms, best_tc = tc;
    }
    h->tune.rotate_tc = best_tc;
    cache[key] = best_tc ? "tc" : "cuda";
    ++tuned;
    return DEREK_OK;
  }

  int jacobi() {
    const std::string key = "jacobi nb=" + std::to_string(h->max_nb_band) + " nks=" + std::to_string(h->nks);
    std::string v;
    if (lookup(key, v) && (v == "pair" || v == "single")) {
      h->tune.jacobi_single = v == "single";
      ++cached;
      return DEREK_OK;
    }
    // a Hermitian Rayleigh quotient of the start vectors: X^H H X
    overlap_all(h, h->d_X, h->d_HX, h->d_Hs, 1);
    float best = 1e30f;
    int best_single = 0;
    for (int single = 0; single <= 1; ++single) {
      const float ms = tm.best(h, 2, [&] {
        launch_jacobi(h->tab_band, 0, h->nks, h->max_nb_band, h->d_Hs, h->d_C, h->d_mat_off, h->d_eig,
                      h->d_scratch, 30, h->prec == DEREK_PREC_FP64 ? 1e-14 : 1e-10, 0, h->d_sweeps, h->stream,
                      single);
      });
      if (ms < best) best = ms, best_single = single;
    }
    h->tune.jacobi_single = best_single;
    cache[key] = best_single ? "single" : "pair";
    ++tuned;
    return DEREK_OK;
  }
};

std::string plan_json(const derek_gpu *h) {
  std::ostringstream o;
  o << "{\"source\": " << quote(h->tune.source) << ", \"fft_radices\": {";
  std::set<int> done;
  bool first = true;
  for (const auto &S : h->sys)
    for (int i = 0; i < 3; ++i)
      if (done.insert(S.plan[i].n).second) {
        o << (first ? "" : ", ") << "\"" << S.plan[i].n << "\": " << quote(radix_str(S.plan[i]));
        first = false;
      }
  o << "}, \"lines\": ";
  if (h->tune.generic_lines) {
    o << "{";
    done.clear();
    first = true;
    for (const auto &S : h->sys)
      for (int i = 0; i < 3; ++i)
        if (done.insert(S.lp[i].n).second) {
          o << (first ? "" : ", ") << "\"" << S.lp[i].n << "\": \"" << S.lp[i].a << "x" << S.lp[i].b << "\"";
          first = false;
        }
    o << "}";
  } else {
    o << "\"" << (h->prec == DEREK_PREC_FP64 ? "fixed-length shared-memory kernels" : "register-line kernels")
      << "\"";
  }
  o << ", \"rows\": {";
  first = true;
  for (const auto &c : h->classes) {
    const int n = c.n[0];
    const char *name = c.disp_m <= c.max_m ? "tight" : (c.disp_m < n / 2 ? "compact" : "all");
    o << (first ? "" : ", ") << "\"" << c.n[0] << "x" << c.n[1] << "x" << c.n[2] << "\": \"" << name << "\"";
    first = false;
  }
  o << "}, \"hpsi_chunk\": " << h->tune.hpsi_chunk;
  o << ", \"overlap\": \"" << (use_tc_overlap(h) ? "tc" : "cuda") << " ksplit " << h->tune.ksplit
    << "\", \"rotate\": \"" << (use_tc_rotate(h) ? "tc" : "cuda") << "\", \"jacobi\": \""
    << (h->tune.jacobi_single ? "single" : "pair") << "\"}";
  return o.str();
}

}  // namespace

extern "C" {

int derek_gpu_autotune(derek_gpu_t *h, const char *cache_path, int flags) {
  if (!h) return DEREK_ERR_BAD_ARG;
  if (reject_spinor(h, "autotune")) return DEREK_ERR_UNSUPPORTED;
  Cache all;
  if (cache_path && *cache_path) {
    std::ifstream f(cache_path);
    if (f) {
      std::stringstream ss;
      ss << f.rdbuf();
      if (!parse_cache(ss.str(), all)) {
        h->last_error = std::string("autotune: cannot parse cache ") + cache_path;
        return DEREK_ERR_BAD_ARG;
      }
    }
  }
  const std::string dev = device_key();
  Tuner t{h, all[dev], !(flags & DEREK_TUNE_RETUNE)};
  // realistic operands: the SCF's start vectors in X, their H psi in HX
  for (auto &S : h->sys) S.active = 1;
  if (int st = upload_sys(h)) return st;
  const int *pw = h->opts.init_vectors == 1 ? h->d_pw_entry : nullptr;
  if (h->prec == DEREK_PREC_FP64)
    launch_init_psi<double>(h->tab, h->nitems, h->d_X, h->opts.seed, pw, h->stream);
  else
    launch_init_psi<float>(h->tab, h->nitems, h->d_X, h->opts.seed, pw, h->stream);
  h->cur = 0;
  int st = DEREK_OK;
  if (!st) st = t.fft_radices();
  if (!st) st = t.lines();
  if (!st) st = t.rows();
  if (!st) st = t.chunks();
  if (!st) st = apply_h_items(h, 0, h->nitems, h->d_X, nullptr, h->d_HX, nullptr);
  if (!st) st = t.overlap();
  if (!st) st = t.jacobi();
  if (!st) st = t.rotate();
  if (st) return st;
  DEREK_CUDA(h, cudaStreamSynchronize(h->stream));
  DEREK_CUDA(h, cudaGetLastError());
  // a tensor-core wait that timed out while timing would have left a status
  DEREK_CUDA(h, cudaMemset(h->d_status, 0, h->nks * sizeof(int)));
  // graphs captured before hold the old plan
  for (auto &g : h->graph_exec)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
  h->graph_degree = -1;
  h->scf_started = false;
  h->tune.source = t.tuned ? (t.cached ? "tuned+cache" : "tuned") : "cache";
  if (cache_path && *cache_path && t.tuned) {
    std::ofstream f(cache_path);
    f << write_cache(all);
    if (!f) {
      h->last_error = std::string("autotune: cannot write cache ") + cache_path;
      return DEREK_ERR_BAD_ARG;
    }
  }
  return DEREK_OK;
}

int derek_gpu_plan(derek_gpu_t *h, char *buf, int len) {
  if (!h || !buf || len <= 0) return DEREK_ERR_BAD_ARG;
  const std::string s = plan_json(h);
  if ((int)s.size() >= len) {
    h->last_error = "plan: buffer too small (" + std::to_string(s.size() + 1) + " bytes needed)";
    return DEREK_ERR_BAD_ARG;
  }
  std::memcpy(buf, s.c_str(), s.size() + 1);
  return DEREK_OK;
}

// host-only: the cache reader/writer and the radix candidates, for checks
// without a GPU
int derek_host_tune_cache_normalise(const char *text, char *out, int len) {
  if (!text || !out || len <= 0) return DEREK_ERR_BAD_ARG;
  Cache c;
  if (!parse_cache(text, c)) return DEREK_ERR_BAD_ARG;
  const std::string s = write_cache(c);
  if ((int)s.size() >= len) return DEREK_ERR_BAD_ARG;
  std::memcpy(out, s.c_str(), s.size() + 1);
  return DEREK_OK;
}

int derek_host_radix_candidates(int n, char *out, int len) {
  if (n <= 0 || !out || len <= 0) return DEREK_ERR_BAD_ARG;
  std::string s;
  for (const auto &c : radix_candidates(n)) s += (s.empty() ? "" : ";") + c;
  if ((int)s.size() >= len) return DEREK_ERR_BAD_ARG;
  std::memcpy(out, s.c_str(), s.size() + 1);
  return DEREK_OK;
}

}  // extern "C"
