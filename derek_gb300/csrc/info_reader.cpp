// A DEReK .info parameter file read the way the reference reads it
// (Source/io.f90 io_read_param 360-830, io_freeform_read 836-882,
// io_block_parse 1765-1937, io_spell_check / io_levenshtein 2545-2630, and
// the conversions of io_initialise 299-353 with Source/units.f90 and the
// CODATA 2018 constants of Source/constants.f90:70-104).
//
// Lines are taken 60 characters at a time (io.f90:382); blank lines and
// lines containing '!' anywhere are skipped; a line holding "$data" opens a
// block; otherwise the text before the first ':' or '=' is the key and the
// rest the value, each kept to 30 characters.  Keys are lower-cased, and so
// are values except for keys containing "unit".  A key within Levenshtein
// distance 1-2 of a known key is corrected to it (the first closest), 3 or
// more is an error.  Values are read list-directed.  Block lines whose
// first character is blank, '#' or '!' are comments; lattice rows and
// potential rows are converted with the units set by the lines above the
// block.
#include <algorithm>
#include <cctype>
#include <cstddef>
#include <cstdlib>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "derek_gpu.h"

namespace {

// ---- units (Source/units.f90:36-127, 208-470): value of one unit in atomic units
struct Si {
  static constexpr double c = 299792458.0, h = 6.62607015e-34, e = 1.602176634e-19, me = 9.1093837015e-31,
                          na = 6.02214076e23, r = 8.314462618;
  static constexpr double pi = 3.141592653589793238462643383279502884197;
};
struct Units {
  double twopi, fourpi, hbar, mu0, eps0, alpha, kb, metre, joule, ev, invmetre;
  Units() {
    twopi = 2.0 * Si::pi;
    fourpi = 4.0 * Si::pi;
    hbar = Si::h / twopi;
    mu0 = fourpi * 1.0E-7;
    eps0 = 1.0 / (mu0 * (Si::c * Si::c));
    alpha = (Si::e * Si::e) / (4.0 * Si::pi * eps0 * hbar * Si::c);
    kb = Si::r / Si::na;
    metre = Si::me * Si::c * alpha / hbar;
    joule = 1.0 / ((alpha * alpha) * Si::me * (Si::c * Si::c));
    ev = Si::e / ((alpha * alpha) * Si::me * (Si::c * Si::c));
    invmetre = 1.0 / metre;
  }
  bool value(const std::string &u, double &v) const {
    const double angstrom = metre * 1e-10, hertz = Si::h * joule;
    struct Entry {
      const char *name;
      double v;
    } table[] = {
        {"bohr", 1.0},
        {"m", metre},
        {"cm", metre * 1e-2},
        {"mm", metre * 1e-3},
        {"mum", metre * 1e-6},
        {"nm", metre * 1e-9},
        {"A", angstrom},
        {"pm", metre * 1e-12},
        {"Ha", 1.0},
        {"mHa", 1e-3},
        {"eV", ev},
        {"meV", ev * 1e-3},
        {"Ry", 0.5},
        {"mRy", 0.5 * 1e-3},
        {"J", joule},
        {"Hz", hertz},
        {"MHz", hertz * 1e6},
        {"GHz", hertz * 1e9},
        {"THz", hertz * 1e12},
        {"cm-1", hertz * Si::c * 1e2},
        {"K", kb * joule},
        {"T", Si::e * (invmetre * invmetre) * twopi / Si::h},
        {"G", 1.0e-4 * Si::e * (invmetre * invmetre) * twopi / Si::h},
        {"agr", 1.0},
        {"Ha/Bohr/e", 1.0},
        {"eV/A/e", ev / angstrom},
        {"N/C", joule / (metre / Si::e)},
    };
    for (const auto &x : table)
      if (u == x.name) {
        v = x.v;
        return true;
      }
    return false;
  }
};

std::string lower(std::string s) {
  for (auto &ch : s) ch = (char)std::tolower((unsigned char)ch);
  return s;
}
std::string rtrim(const std::string &s) {
  size_t e = s.size();
  while (e > 0 && s[e - 1] == ' ') --e;
  return s.substr(0, e);
}
std::string adjustl_trim(const std::string &s) {
  size_t b = 0;
  while (b < s.size() && s[b] == ' ') ++b;
  return rtrim(s.substr(b));
}
std::string fixed(const std::string &s, size_t n) { return s.size() > n ? s.substr(0, n) : s; }

int levenshtein(const std::string &a, const std::string &b) {
  std::vector<std::vector<int>> d(a.size() + 1, std::vector<int>(b.size() + 1));
  for (size_t i = 0; i <= a.size(); ++i) d[i][0] = (int)i;
  for (size_t j = 0; j <= b.size(); ++j) d[0][j] = (int)j;
  for (size_t i = 1; i <= a.size(); ++i)
    for (size_t j = 1; j <= b.size(); ++j)
      d[i][j] = std::min({d[i - 1][j] + 1, d[i][j - 1] + 1, d[i - 1][j - 1] + (a[i - 1] == b[j - 1] ? 0 : 1)});
  return d[a.size()][b.size()];
}

// ---- list-directed input of one value string (blank or comma separated;
// r*c repeat counts; '/' ends the input)
struct ListReader {
  std::vector<std::string> items;
  bool slash = false;
  explicit ListReader(const std::string &s) {
    size_t i = 0;
    while (i < s.size() && !slash) {
      while (i < s.size() && (s[i] == ' ' || s[i] == ',')) ++i;
      if (i >= s.size()) break;
      if (s[i] == '/') {
        slash = true;
        break;
      }
      std::string tok;
      if (s[i] == '\'' || s[i] == '"') {   // quoted character value
        const char q = s[i++];
        while (i < s.size()) {
          if (s[i] == q) {
            if (i + 1 < s.size() && s[i + 1] == q) {
              tok += q;
              i += 2;
              continue;
            }
            ++i;
            break;
          }
          tok += s[i++];
        }
        items.push_back(tok);
        continue;
      }
      while (i < s.size() && s[i] != ' ' && s[i] != ',' && s[i] != '/') tok += s[i++];
      const size_t star = tok.find('*');
      if (star != std::string::npos && star > 0 &&
          tok.find_first_not_of("0123456789") == star) {   // r*c
        const int r = std::atoi(tok.substr(0, star).c_str());
        for (int k = 0; k < r; ++k) items.push_back(tok.substr(star + 1));
      } else {
        items.push_back(tok);
      }
    }
  }
};

bool parse_int(const std::string &t, int &v) {
  size_t i = 0;
  if (i < t.size() && (t[i] == '+' || t[i] == '-')) ++i;
  if (i >= t.size()) return false;
  for (size_t j = i; j < t.size(); ++j)
    if (!std::isdigit((unsigned char)t[j])) return false;
  v = std::atoi(t.c_str());
  return true;
}

bool parse_real(const std::string &t, double &v) {
  // [sign] digits [. digits] [ (e|d|q)[sign]digits | sign digits ]
  size_t i = 0;
  std::string m;
  if (i < t.size() && (t[i] == '+' || t[i] == '-')) m += t[i++];
  bool digits = false;
  while (i < t.size() && std::isdigit((unsigned char)t[i])) m += t[i++], digits = true;
  if (i < t.size() && t[i] == '.') {
    m += t[i++];
    while (i < t.size() && std::isdigit((unsigned char)t[i])) m += t[i++], digits = true;
  }
  if (!digits) return false;
  if (i < t.size()) {
    const char c = (char)std::tolower((unsigned char)t[i]);
    if (c == 'e' || c == 'd' || c == 'q') ++i;
    else if (c != '+' && c != '-') return false;
    std::string ex;
    if (i < t.size() && (t[i] == '+' || t[i] == '-')) ex += t[i++];
    size_t nd = 0;
    while (i < t.size() && std::isdigit((unsigned char)t[i])) ex += t[i++], ++nd;
    if (nd == 0 || i != t.size()) return false;
    m += "e" + ex;
  }
  v = std::strtod(m.c_str(), nullptr);
  return true;
}

bool parse_logical(const std::string &t, int &v) {
  size_t i = 0;
  if (i < t.size() && t[i] == '.') ++i;
  if (i >= t.size()) return false;
  const char c = (char)std::tolower((unsigned char)t[i]);
  if (c == 't') v = 1;
  else if (c == 'f') v = 0;
  else return false;
  return true;
}

void set_str(char *dst, const std::string &s) {
  const std::string x = fixed(s, 30);
  std::memset(dst, 0, 32);
  std::memcpy(dst, x.data(), x.size());
}

enum Kind { LOGICAL, INT, REAL, STR, INT3, REAL3 };
struct Key {
  const char *name;
  Kind kind;
  size_t off;
};

#define K(n, k, f) {n, k, offsetof(derek_info, f)}
const Key kKeys[] = {   // Source/io.f90:116-162 and keys_array 1281-1325
    K("check", LOGICAL, check),
    K("profilling", LOGICAL, debugging),
    K("n_electrons", INT, n_electrons),
    K("energy_tol", REAL, energy_tol),
    K("xc_functional", STR, xc_functional),
    K("cut_off_energy", REAL, cut_off_energy),
    K("g_fine_scale", REAL, g_fine_scale),
    K("write_wvfn", LOGICAL, write_wvfn),
    K("task", STR, task),
    K("soc", LOGICAL, soc),
    K("max_scf", INT, max_scf),
    K("scf_method", STR, scf_method),
    K("electronic_temp", REAL, electronic_temp),
    K("conduction_bands", INT, conduction_bands),
    K("write_density", LOGICAL, write_density),
    K("write_potential", LOGICAL, write_potential),
    K("write_state", LOGICAL, write_state),
    K("external_pot", STR, external_pot),
    K("kpt_mp_grid", INT3, kpt_mp_grid),
    K("write_spec", LOGICAL, write_spec),
    K("write_memory", LOGICAL, write_memory),
    K("print_level", INT, iprint),
    K("finite_barrier_height", REAL, finite_barrier_height),
    K("finite_barrier_width", REAL3, finite_barrier_width),
    K("periodic_pot_grid", INT3, periodic_pot_grid),
    K("periodic_pot_amp", REAL, periodic_pot_amp),
    K("random_seed", INT, random_seed),
    K("write_formatted_potential", LOGICAL, write_formatted_potential),
    K("write_potex", LOGICAL, write_potex),
    K("write_formatted_density", LOGICAL, write_formatted_density),
    K("write_formatted_potex", LOGICAL, write_formatted_potex),
    K("output_level", STR, output_level),
    K("ext_efield", REAL3, ext_efield),
    K("ext_bfield", REAL3, ext_bfield),
    K("unit_energy", STR, unit_energy),
    K("unit_length", STR, unit_length),
    K("unit_efield", STR, unit_efield),
    K("unit_bfield", STR, unit_bfield),
    K("unit_energy_out", STR, out_energy_unit),
    K("unit_length_out", STR, out_len_unit),
    K("unit_efield_out", STR, out_efield_unit),
    K("unit_bfield_out", STR, out_bfield_unit),
    K("lattice", STR, task),   // keys_array(43): a block name, no value key
    K("dos_kpt_mp_grid", INT3, dos_kpt_mp_grid),
    K("write_xsf", LOGICAL, write_xsf),
};
#undef K

void defaults(derek_info &p) {   // Source/io.f90:63-110
  std::memset(&p, 0, sizeof p);
  p.n_electrons = 1;
  p.energy_tol = 1.0E-7;
  set_str(p.xc_functional, "LDA");
  p.cut_off_energy = 200.0;
  p.g_fine_scale = 2.0;
  set_str(p.task, "singlepoint");
  p.max_scf = 40;
  set_str(p.scf_method, "EDFT");
  p.electronic_temp = 0.0;
  p.conduction_bands = 20;
  p.write_state = 1;
  set_str(p.external_pot, "jelly");
  for (int i = 0; i < 3; ++i) {
    p.kpt_mp_grid[i] = 1;
    p.periodic_pot_grid[i] = 1;
    p.dos_kpt_mp_grid[i] = 11;
    p.finite_barrier_width[i] = 0.5;
  }
  p.write_spec = 1;
  p.iprint = 1;
  p.finite_barrier_height = 10.00;
  p.periodic_pot_amp = 10.00;
  set_str(p.output_level, "minimal");
  set_str(p.unit_energy, "eV");
  set_str(p.unit_length, "A");
  set_str(p.unit_efield, "eV/A/e");
  set_str(p.unit_bfield, "T");
  set_str(p.out_energy_unit, "eV");
  set_str(p.out_len_unit, "A");
  set_str(p.out_efield_unit, "eV/A/e");
  set_str(p.out_bfield_unit, "G");
}

struct Fail {
  std::string msg;
};

bool file_exists(const std::string &p) {
  FILE *f = std::fopen(p.c_str(), "r");
  if (!f) return false;
  std::fclose(f);
  return true;
}

}  // namespace

extern "C" int derek_info_read(const char *path, derek_info *out, char *message, int message_len) {
  if (!path || !out) return DEREK_ERR_BAD_ARG;
  derek_info p;
  defaults(p);
  const Units units;
  auto to_atomic = [&](double x, const char *unit) {
    double v;
    if (!units.value(unit, v)) throw Fail{std::string("Unknown unit: ") + unit};
    return x * v;
  };
  std::string note;
  try {
    std::ifstream in(path);
    if (!in) throw Fail{std::string("cannot open ") + path};
    std::vector<std::string> lines;
    for (std::string l; std::getline(in, l);) {
      if (!l.empty() && l.back() == '\r') l.pop_back();
      lines.push_back(l);
    }
    std::vector<std::string> present;
    bool cell_declared = false;
    for (size_t i = 0; i < lines.size(); ++i) {
      const std::string line = rtrim(fixed(lines[i], 60));
      if (line.empty()) continue;
      if (line.find('!') != std::string::npos) continue;
      if (lower(line).find("$data") != std::string::npos) {
        const std::string ext_before = p.external_pot;
        ListReader hdr(adjustl_trim(lower(line)));
        if (hdr.items.size() < 2) throw Fail{" problem parsing block"};
        const std::string type_in = fixed(hdr.items[1], 20);
        size_t j = i + 1;
        for (;; ++j) {
          if (j >= lines.size()) throw Fail{"Block " + type_in + " not closed"};
          const std::string b = adjustl_trim(lower(fixed(lines[j], 300)));
          if (b.find("$enddata") != std::string::npos) {
            ListReader end(b);
            if (end.items.size() < 2) throw Fail{"Problem parsing end block"};
            if (fixed(end.items[1], 20) != type_in) throw Fail{"Block " + type_in + " not closed"};
            break;
          }
        }
        std::vector<std::string> data;
        for (size_t k = i + 1; k < j; ++k) {
          const std::string b = fixed(lines[k], 300);
          if (b.empty() || b[0] == '#' || b[0] == '!' || b[0] == ' ') continue;   // comments
          data.push_back(b);
        }
        if (data.empty()) throw Fail{"No data in block"};
        if (type_in == "lattice") {
          if (data.size() != 3) throw Fail{"LATTICE must have 3 lines"};
          for (int r = 0; r < 3; ++r) {
            ListReader lr(data[r]);
            double v[3];
            if (lr.items.size() < 3 || !parse_real(lr.items[0], v[0]) || !parse_real(lr.items[1], v[1]) ||
                !parse_real(lr.items[2], v[2]))
              throw Fail{"Error parsing lattice matrix"};
            for (int c = 0; c < 3; ++c) p.cell[r + 3 * c] = to_atomic(v[c], p.unit_length);
          }
          cell_declared = true;
        } else if (type_in == "gaussian_pot" || type_in == "lorentzian_pot") {
          set_str(p.external_pot, type_in);
          if (data.size() > 64) throw Fail{"more than 64 potential rows"};
          p.n_pots = (int)data.size();
          for (size_t r = 0; r < data.size(); ++r) {
            ListReader lr(data[r]);
            double v[5];
            if (lr.items.size() < 5) throw Fail{"Error parsing potential block"};
            for (int c = 0; c < 5; ++c)
              if (!parse_real(lr.items[c], v[c])) throw Fail{"Error parsing potential block"};
            for (int c = 0; c < 3; ++c) p.pot_centres[3 * r + c] = v[c];
            p.pot_heights[r] = to_atomic(v[3], p.unit_energy);
            p.pot_widths[r] = to_atomic(v[4], p.unit_length);
          }
        } else {
          throw Fail{" Unknown block type " + type_in};
        }
        if (std::string(p.external_pot) != ext_before) present.push_back("external_pot");
        i = j;   // the close line is consumed
        continue;
      }
      if (line[0] == '!' || line[0] == '#') continue;
      const size_t sep = line.find_first_of(":=");
      if (sep == std::string::npos) throw Fail{" Error parsing line:  " + line};
      std::string key = adjustl_trim(lower(fixed(line.substr(0, sep), 30)));
      std::string val = fixed(line.substr(sep + 1), 30);
      if (key.find("unit") == std::string::npos) val = adjustl_trim(lower(val));
      // spell check: the first closest key (Source/io.f90:2593-2630)
      int best = 1 << 30;
      const Key *match = nullptr;
      for (const auto &k : kKeys) {
        const int d = levenshtein(key, k.name);
        if (d < best) {
          best = d;
          match = &k;
        }
      }
      if (best >= 3) throw Fail{"Unknown parameter - " + key};
      if (best > 0) {
        note += key + " -> " + match->name + "; ";
        ++p.n_corrected;
      }
      key = match->name;
      if (key == "lattice") throw Fail{" Error parsing keyword: " + key};
      ListReader lr(val);
      char *base = reinterpret_cast<char *>(&p) + match->off;
      const std::string bad = " Error parsing value: " + val;
      // item n, or nullptr when a '/' ended the record before it (the
      // variable keeps its value); running out without a '/' is an error
      auto item = [&](size_t n) -> const std::string * {
        if (n < lr.items.size()) return &lr.items[n];
        if (lr.slash) return nullptr;
        throw Fail{bad};
      };
      const int count = match->kind == INT3 || match->kind == REAL3 ? 3 : 1;
      for (int c = 0; c < count; ++c) {
        const std::string *t = item((size_t)c);
        if (!t) break;
        bool ok = true;
        switch (match->kind) {
          case LOGICAL: ok = parse_logical(*t, *reinterpret_cast<int *>(base)); break;
          case INT: ok = parse_int(*t, *reinterpret_cast<int *>(base)); break;
          case REAL: ok = parse_real(*t, *reinterpret_cast<double *>(base)); break;
          case STR: set_str(base, *t); break;
          case INT3: ok = parse_int(*t, reinterpret_cast<int *>(base)[c]); break;
          case REAL3: ok = parse_real(*t, reinterpret_cast<double *>(base)[c]); break;
        }
        if (!ok) throw Fail{bad};
      }
      if (key == "task") {
        const std::string t = p.task;
        if (t != "singlepoint" && t != "bandstructure" && t != "dos") throw Fail{"Unknown task: " + val};
      } else if (key == "external_pot") {
        const std::string e = p.external_pot;
        if (e == "gaussian_pot" || e == "lorentzian_pot")
          throw Fail{"External pot type " + e + " should only be set in a data block."};
        if (e != "jelly" && e != "finite_barrier" && e != "periodic_pot") {
          if (!file_exists(e)) throw Fail{"Potential file does not exist: " + e};
          if (e.find("potex") == std::string::npos) throw Fail{"Unsupported external potential file: " + e};
        }
      } else if (key == "print_level") {
        if (p.iprint < 1 || p.iprint > 3) throw Fail{"print_level  must be between 1 and 3"};
      }
      present.push_back(key);
    }
    for (size_t a = 0; a < present.size(); ++a)
      for (size_t b = 0; b < present.size(); ++b)
        if (a != b && present[a] == present[b]) throw Fail{" Duplicate parameter found: " + present[a]};
    // write flags of output_level (Source/io.f90:782-819)
    for (const auto &k : present)
      if (k == "output_level") {
        const std::string o = p.output_level;
        int *flags[] = {&p.write_wvfn, &p.write_spec, &p.write_state, &p.write_potex, &p.write_formatted_potex,
                        &p.write_density, &p.write_formatted_density, &p.write_potential,
                        &p.write_formatted_potential};
        if (o == "minimal") {
          const int v[] = {0, 0, 1, 1, 0, 1, 0, 0, 0};
          for (int q = 0; q < 9; ++q) *flags[q] = v[q];
        } else if (o == "none") {
          for (int q = 0; q < 9; ++q) *flags[q] = 0;
        } else if (o == "all") {
          for (int q = 0; q < 9; ++q) *flags[q] = 1;
        }
      }
    if (std::string(p.task) == "bandstructure" || std::string(p.task) == "dos") p.write_spec = 1;
    if (!cell_declared) throw Fail{" No lattice provided"};
    // io_initialise (Source/io.f90:316, 338-353)
    p.nbands = p.n_electrons + p.conduction_bands;
    p.energy_tol = to_atomic(p.energy_tol, p.unit_energy);
    p.cut_off_energy = to_atomic(p.cut_off_energy, p.unit_energy);
    p.electronic_temp = to_atomic(p.electronic_temp, "K");
    p.finite_barrier_height = to_atomic(p.finite_barrier_height, p.unit_energy);
    for (int c = 0; c < 3; ++c) p.finite_barrier_width[c] = to_atomic(p.finite_barrier_width[c], p.unit_length);
    p.periodic_pot_amp = to_atomic(p.periodic_pot_amp, p.unit_energy);
    for (int c = 0; c < 3; ++c) p.ext_efield[c] = to_atomic(p.ext_efield[c], p.unit_efield);
    for (int c = 0; c < 3; ++c) p.ext_bfield[c] = to_atomic(p.ext_bfield[c], p.unit_bfield);
  } catch (const Fail &f) {
    if (message && message_len > 0) std::snprintf(message, (size_t)message_len, "%s", f.msg.c_str());
    return DEREK_ERR_BAD_ARG;
  }
  if (message && message_len > 0) std::snprintf(message, (size_t)message_len, "%s", note.c_str());
  *out = p;
  return DEREK_OK;
}
