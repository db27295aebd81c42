// Input decks and output formats of HeatFlow (see deck.hpp for the reference routines followed).
#include "deck.hpp"

#include <algorithm>
#include <cctype>
#include <cerrno>
#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <sstream>
#include <sys/stat.h>

namespace hfhost {
namespace {

std::string trim(const std::string& s) {
  size_t a = 0, b = s.size();
  while (a < b && std::isspace((unsigned char)s[a])) ++a;
  while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
  return s.substr(a, b - a);
}

std::vector<std::string> split_ws(const std::string& s) {
  std::vector<std::string> out;
  size_t i = 0;
  while (i < s.size()) {
    while (i < s.size() && std::isspace((unsigned char)s[i])) ++i;
    size_t j = i;
    while (j < s.size() && !std::isspace((unsigned char)s[j])) ++j;
    if (j > i) out.push_back(s.substr(i, j - i));
    i = j;
  }
  return out;
}

std::vector<std::string> split_lines(const std::string& text) {
  std::vector<std::string> out;
  std::string cur;
  for (size_t i = 0; i < text.size(); ++i) {
    const char ch = text[i];
    if (ch == '\n' || ch == '\r') {
      out.push_back(cur);
      cur.clear();
      if (ch == '\r' && i + 1 < text.size() && text[i + 1] == '\n') ++i;
    } else {
      cur.push_back(ch);
    }
  }
  if (!cur.empty()) out.push_back(cur);
  return out;
}

std::string rstrip_commas(std::string s) {
  while (!s.empty() && s.back() == ',') s.pop_back();
  return s;
}

// A Fortran real token: 1.5d-3 and 1.5e-3 alike, trailing commas ignored.
double fortran_real(const std::string& tok) {
  std::string t = rstrip_commas(trim(tok));
  for (char& ch : t) {
    if (ch == 'd') ch = 'e';
    if (ch == 'D') ch = 'E';
  }
  if (t.empty()) throw InputError("Error: empty number");
  char* end = nullptr;
  errno = 0;
  const double v = std::strtod(t.c_str(), &end);
  if (end != t.c_str() + t.size()) throw InputError("Error: not a number: " + tok);
  return v;
}

int64_t fortran_int(const std::string& tok) {
  const std::string t = rstrip_commas(trim(tok));
  if (t.empty()) throw InputError("Error: empty integer");
  char* end = nullptr;
  const long long v = std::strtoll(t.c_str(), &end, 10);
  if (end != t.c_str() + t.size()) throw InputError("Error: not an integer: " + tok);
  return (int64_t)v;
}

std::string strip_comment(const std::string& line) {
  const size_t k = line.find('!');
  return k == std::string::npos ? line : line.substr(0, k);
}

// (keyword, value) as assignD/I/L/S see them: the keyword is the text before the first '=', the
// value the text after the last '=' (val, mod_inputs.f90:819-826).
bool keyword_value(const std::string& line, std::string& key, std::string& value) {
  const size_t a = line.find('='), b = line.rfind('=');
  if (a == std::string::npos) return false;
  key = trim(line.substr(0, a));
  value = trim(line.substr(b + 1));
  return true;
}

bool contains(const std::string& s, const char* sub) { return s.find(sub) != std::string::npos; }

bool is_integer_token(const std::string& s) {
  size_t i = 0;
  if (i < s.size() && (s[i] == '+' || s[i] == '-')) ++i;
  if (i == s.size()) return false;
  for (; i < s.size(); ++i)
    if (!std::isdigit((unsigned char)s[i])) return false;
  return true;
}

// read_param's keywords in readvar order (mod_inputs.f90:283-327).
enum Kind { KI, KD, KL, KS };
struct Key {
  const char* name;
  Kind kind;
};
const Key kParamKeys[] = {
    {"IVERB", KI}, {"ntime", KI}, {"time_step", KD}, {"freq", KD}, {"iboundary", KI},
    {"icattaneo", KI}, {"isteady", KI}, {"power_in", KD}, {"kappaBoundx1", KD},
    {"kappaBoundy1", KD}, {"kappaBoundz1", KD}, {"_Check_Sparse_Full", KL},
    {"_Check_Stability", KL}, {"_WriteToTxt", KL}, {"_Percentage_Completion", KL},
    {"_Test_Run", KL}, {"_InputTempDis", KL}, {"_RunName", KS}, {"_FullRestart", KL},
    {"T_Bathx1", KD}, {"T_Bathx2", KD}, {"T_Bathy1", KD}, {"T_Bathy2", KD}, {"T_Bathz1", KD},
    {"T_Bathz2", KD}, {"T_System", KD}, {"T_Bath", KD}, {"kappaBound", KD}, {"kappaBoundNx", KD},
    {"kappaBoundNy", KD}, {"kappaBoundNz", KD}, {"start_ix", KI}, {"end_ix", KI},
    {"start_iy", KI}, {"end_iy", KI}, {"start_iz", KI}, {"end_iz", KI}, {"write_every", KI},
    {"TempDepProp", KI}, {"Periodic", KS}, {"heattime", KI}, {"T_BathCG", KD}, {"BR", KD},
    {"T_BathCC", KL}, {"CG_dir", KS},
};
constexpr int kNParam = (int)(sizeof(kParamKeys) / sizeof(kParamKeys[0]));

void* param_slot(Param& p, int idx) {
  switch (idx) {
    case 0: return &p.iverb;
    case 1: return &p.ntime;
    case 2: return &p.time_step;
    case 3: return &p.freq;
    case 4: return &p.iboundary;
    case 5: return &p.icattaneo;
    case 6: return &p.isteady;
    case 7: return &p.power_in;
    case 8: return &p.kb[0];
    case 9: return &p.kb[2];
    case 10: return &p.kb[4];
    case 11: return &p.check_sparse_full;
    case 12: return &p.check_stability;
    case 13: return &p.write_to_txt;
    case 14: return &p.percentage_completion;
    case 15: return &p.test_run;
    case 16: return &p.input_temp_dis;
    case 17: return &p.run_name;
    case 18: return &p.full_restart;
    case 19: return &p.t_bath_face[0];
    case 20: return &p.t_bath_face[1];
    case 21: return &p.t_bath_face[2];
    case 22: return &p.t_bath_face[3];
    case 23: return &p.t_bath_face[4];
    case 24: return &p.t_bath_face[5];
    case 25: return &p.t_system;
    case 26: return &p.t_bath;
    case 27: return &p.kappa_bound;
    case 28: return &p.kb[1];
    case 29: return &p.kb[3];
    case 30: return &p.kb[5];
    case 31: return &p.start_ix;
    case 32: return &p.end_ix;
    case 33: return &p.start_iy;
    case 34: return &p.end_iy;
    case 35: return &p.start_iz;
    case 36: return &p.end_iz;
    case 37: return &p.write_every;
    case 38: return &p.temp_dep_prop;
    case 39: return &p.periodic_text;
    case 40: return &p.heattime;
    case 41: return &p.t_bath_cg;
    case 42: return &p.br;
    case 43: return &p.t_bath_cc;
    case 44: return &p.cg_dir;
    default: return nullptr;
  }
}

// check_param (mod_inputs.f90:366-596): warnings are silent, errors throw.
void check_param(Param& p, std::vector<int>& rv) {
  for (int v : rv)
    if (v > 1) throw InputError("ERROR: same KEYWORD apears more than once");
  const int kb[3] = {rv[8], rv[9], rv[10]}, kbn[3] = {rv[28], rv[29], rv[30]};
  auto has0 = [](const int* a) { return a[0] == 0 || a[1] == 0 || a[2] == 0; };
  auto all1 = [](const int* a) { return a[0] == 1 && a[1] == 1 && a[2] == 1; };
  if (!(p.periodic[0] && p.periodic[1] && p.periodic[2])) {
    if ((has0(kb) || has0(kbn)) && rv[27] == 0)
      throw InputError("ERROR: KappaBoundx,y,z and KappaBound are not set");
    if ((all1(kb) || all1(kbn)) && rv[27] == 0) rv[27] = 1;
    if ((has0(kb) || has0(kbn)) && rv[27] == 1)
      for (double& k : p.kb) k = p.kappa_bound;
  }
  if (rv[41] == 1 && p.t_bath_cg > 0) {
    for (int k = 19; k < 25; ++k) rv[k] = 1;
    rv[26] = 1;
  }
  bool face_missing = false;
  for (int k = 19; k < 25; ++k) face_missing |= rv[k] == 0;
  if (face_missing)
    for (double& t : p.t_bath_face) t = p.t_bath;
  if (rv[41] == 0) p.t_bath_cg = 0.0;
}

struct Builtin {
  int64_t index;
  double heat_capacity, h_conv, kappa, kappa3D, rho, sound_speed, tau;
};
// Built-in materials, mod_material.f90:116-265 (tau and em are 0 where the reference leaves them).
const Builtin kBuiltin[] = {
    {100, 1.0, 21.4, 1.0, 0.02587, 1.0, 0.0, 0.0},
    {140, 4200.0, 0.0, 130.0, 130.0, 2328.0, 8433.0, 0.0},
    {3001, 840.0, 0.0, 0.19, 0.19, 941.0, 1000.0, 0.0},
    {3002, 1100.0, 0.0, 1.42, 1.42, 1700.0, 1000.0, 0.0},
    {3003, 1400.0, 0.0, 1.59, 1.59, 1800.0, 1000.0, 0.0},
    {3004, 2300.0, 0.0, 1.25, 1.25, 2300.0, 1000.0, 0.0},
    {9001, 3421.0, 0.0, 0.6, 0.0, 1090.0, 3.0, 0.0},
    {9002, 3391.0, 0.0, 0.209, 0.0, 1109.0, 3.0, 0.0},
    {9003, 2348.0, 0.0, 0.317, 0.0, 911.0, 3.0, 0.0},
    {310, 700.0, 0.0, 130.0, 130.0, 2329.0, 8433.0, 0.0},
    {320, 720.0, 0.0, 1.4, 1.4, 2400.0, 5970.0, 1.0},
    {330, 236.0, 0.0, 427.0, 429.0, 10524.0, 3650.0, 0.0},
    {340, 1500.0, 0.0, 0.2, 0.2, 1153.0, 8433.0, 1.0},
    {350, 361.0, 0.0, 10.2, 10.2, 7140.0, 3650.0, 1.0},
};

std::string es16_8(double v) {
  char buf[64];
  std::snprintf(buf, sizeof(buf), "%16.8E", v);
  return buf;
}

void append_json_array(std::ostringstream& o, const char* name, const double* v, int64_t n) {
  o << "\"" << name << "\": [";
  char buf[40];
  for (int64_t i = 0; i < n; ++i) {
    std::snprintf(buf, sizeof(buf), "%.17g", v[i]);
    o << (i ? ", " : "") << buf;
  }
  o << "]";
}

std::string json_num(double v) {
  char buf[40];
  std::snprintf(buf, sizeof(buf), "%.17g", v);
  return buf;
}

}  // namespace

Param read_param(const std::string& text) {
  Param p;
  std::vector<int> rv(kNParam, 0);
  for (const std::string& raw : split_lines(text)) {
    const std::string line = strip_comment(raw);
    if (trim(line).empty()) continue;
    std::string key, value;
    if (!keyword_value(line, key, value) || value.empty()) continue;
    for (int idx = 0; idx < kNParam; ++idx) {
      if (key != kParamKeys[idx].name) continue;
      rv[idx] += 1;
      void* slot = param_slot(p, idx);
      const std::vector<std::string> toks = split_ws(value);
      switch (kParamKeys[idx].kind) {
        case KI: *static_cast<int64_t*>(slot) = fortran_int(toks.at(0)); break;
        case KD: *static_cast<double*>(slot) = fortran_real(toks.at(0)); break;
        case KL:
          if (contains(value, "T") || contains(value, "t")) *static_cast<bool*>(slot) = true;
          if (contains(value, "F") || contains(value, "f")) *static_cast<bool*>(slot) = false;
          break;
        case KS: *static_cast<std::string*>(slot) = toks.empty() ? std::string() : toks[0]; break;
      }
    }
  }
  const std::string& per = p.periodic_text;
  p.periodic[0] = contains(per, "x") || contains(per, "X");
  p.periodic[1] = contains(per, "y") || contains(per, "Y");
  p.periodic[2] = contains(per, "z") || contains(per, "Z");
  const char* faces[6] = {"-x", "+x", "-y", "+y", "-z", "+z"};
  for (int f = 0; f < 6; ++f) p.cg[f] = contains(p.cg_dir, faces[f]);
  check_param(p, rv);
  return p;
}

std::vector<Material> read_mat(const std::string& text) {
  static const char* keys[8] = {"heat_capacity", "h_conv", "kappa", "kappa3D",
                                "rho",           "sound_speed", "tau", "em"};
  std::vector<Material> mats;
  int found[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  bool have = false;
  for (const std::string& raw : split_lines(text)) {
    const std::string line = strip_comment(raw);
    if (trim(line).empty()) continue;
    const std::string first = rstrip_commas(split_ws(line).at(0));
    if (is_integer_token(first)) {
      const int64_t idx = fortran_int(first);
      if (idx == 0) {
        bool bad = false;
        for (int v : found) bad |= v != 1;
        if (bad) {
          std::string msg = "Error in parameters : material [";
          for (int k = 0; k < 8; ++k) msg += (k ? ", " : "") + std::to_string(found[k]);
          throw InputError(msg + "]");
        }
        for (int& v : found) v = 0;
      } else {
        Material m;
        m.index = idx;
        mats.push_back(m);
        have = true;
        if (mats.size() == 101) throw InputError("Error: code does not suporrt over 100 materials");
      }
      continue;
    }
    std::string key, value;
    if (!keyword_value(line, key, value) || !have) continue;
    Material& cur = mats.back();
    double* slots[8] = {&cur.heat_capacity, &cur.h_conv, &cur.kappa, &cur.kappa3D,
                        &cur.rho,           &cur.sound_speed, &cur.tau, &cur.em};
    for (int k = 0; k < 8; ++k) {
      if (key == keys[k] && !value.empty()) {
        found[k] += 1;
        *slots[k] = fortran_real(split_ws(value).at(0));
      }
    }
  }
  for (size_t i = 0; i < mats.size(); ++i)
    for (size_t j = 0; j < i; ++j)
      if (mats[i].index == mats[j].index)
        throw InputError("Error: Duplicate material index " + std::to_string(mats[i].index));
  return mats;
}

System read_system(const std::string& text) {
  const std::vector<std::string> lines = split_lines(text);
  if (lines.size() < 2) throw InputError("Error: Unexpected EOF system.in");
  System s;
  {
    const auto t = split_ws(lines[0]);
    if (t.size() < 3) throw InputError("Error: system.in: grid dimensions");
    s.nx = fortran_int(t[0]); s.ny = fortran_int(t[1]); s.nz = fortran_int(t[2]);
    const auto u = split_ws(lines[1]);
    if (u.size() < 3) throw InputError("Error: system.in: box lengths");
    s.lx = fortran_real(u[0]); s.ly = fortran_real(u[1]); s.lz = fortran_real(u[2]);
  }
  if (s.nx < 1 || s.ny < 1 || s.nz < 1) throw InputError("Error: system.in: grid dimensions");
  const int64_t n = s.nx * s.ny * s.nz;
  s.imaterial.assign(n, 0);
  s.iheater.assign(n, 0);
  size_t pos = 2;
  for (int64_t iz = 0; iz < s.nz; ++iz) {
    pos += 1;                                   // the line before each plane
    for (int64_t iy = 0; iy < s.ny; ++iy) {
      if (pos >= lines.size()) throw InputError("Error: Unexpected EOF system.in");
      const auto toks = split_ws(lines[pos]);
      pos += 1;
      if ((int64_t)toks.size() < s.nx) throw InputError("Error: Unexpected EOF system.in");
      for (int64_t ix = 0; ix < s.nx; ++ix) {
        const std::string& tk = toks[ix];
        const size_t c = tk.find(':');
        if (c == std::string::npos || tk.find(':', c + 1) != std::string::npos)
          throw InputError("Error: system.in: expected material:heater, got " + tk);
        const int64_t I = ix + s.nx * (iy + s.ny * iz);
        s.imaterial[I] = fortran_int(tk.substr(0, c));
        s.iheater[I] = fortran_int(tk.substr(c + 1));
      }
    }
  }
  return s;
}

Material material(int64_t imaterial, const std::vector<Material>& mats) {
  const std::string msg = "Error: imaterial_type not recognized: " + std::to_string(imaterial);
  if (imaterial <= 0) throw InputError(msg);
  if (imaterial <= 99) {
    for (const auto& m : mats)
      if (m.index == imaterial) return m;
    throw InputError(msg);
  }
  for (const auto& b : kBuiltin) {
    if (b.index != imaterial) continue;
    Material m;
    m.index = b.index;
    m.heat_capacity = b.heat_capacity; m.h_conv = b.h_conv; m.kappa = b.kappa;
    m.kappa3D = b.kappa3D; m.rho = b.rho; m.sound_speed = b.sound_speed; m.tau = b.tau;
    return m;
  }
  throw InputError(msg);
}

void build_deck(Deck& deck, const std::string& param_text, const std::string& mat_text,
                const std::string& system_text) {
  deck.param = read_param(param_text);
  deck.mats = read_mat(mat_text);
  deck.sys = read_system(system_text);
  const Param& p = deck.param;
  const System& s = deck.sys;
  const int64_t n = deck.ncells();
  deck.kappa.resize(n); deck.rho.resize(n); deck.heat_capacity.resize(n); deck.tau.resize(n);
  deck.em.resize(n);
  std::map<int64_t, Material> cache;
  for (int64_t I = 0; I < n; ++I) {
    const int64_t im = s.imaterial[I];
    auto it = cache.find(im);
    if (it == cache.end()) it = cache.emplace(im, material(im, deck.mats)).first;
    const Material& m = it->second;
    deck.kappa[I] = m.kappa; deck.rho[I] = m.rho; deck.heat_capacity[I] = m.heat_capacity;
    deck.tau[I] = m.tau; deck.em[I] = m.em;
  }
  hf_problem& q = deck.prob;
  q = hf_problem{};
  q.nx = s.nx; q.ny = s.ny; q.nz = s.nz;
  q.lx = s.lx; q.ly = s.ly; q.lz = s.lz;
  q.kappa = deck.kappa.data(); q.rho = deck.rho.data(); q.heat_capacity = deck.heat_capacity.data();
  q.tau = deck.tau.data(); q.em = deck.em.data(); q.iheater = deck.sys.iheater.data();
  q.power = nullptr;
  q.power_in = p.power_in; q.freq = p.freq; q.time_step = p.time_step;
  q.heated_steps = p.heattime; q.icattaneo = (int32_t)p.icattaneo; q.isteady = (int32_t)p.isteady;
  for (int a = 0; a < 3; ++a) q.periodic[a] = p.periodic[a] ? 1 : 0;
  for (int f = 0; f < 6; ++f) {
    q.cg_face[f] = p.cg[f] ? 1 : 0;
    q.kappa_bound[f] = p.kb[f];
    q.t_bath_face[f] = p.t_bath_face[f];
  }
  q.t_bath = p.t_bath; q.t_bath_cg = p.t_bath_cg; q.br = p.br;
  q.qdens_mode = HF_QDENS_HEATED_VOLUME;
}

std::string read_text_file(const std::string& path, const std::string& missing_message) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw InputError(missing_message);
  std::ostringstream o;
  o << f.rdbuf();
  return o.str();
}

std::string format_temp_file(const double* v, int64_t n) {
  std::string out;
  out.reserve((size_t)n * 17 + 8);
  for (int64_t k = 0; k < n; k += 6) {
    for (int64_t i = k; i < std::min<int64_t>(k + 6, n); ++i) out += es16_8(v[i]) + " ";
    out += "\n";
  }
  out += "\n\n";
  return out;
}

std::vector<double> parse_temp_file(const std::string& text, int64_t na) {
  std::vector<double> vals;
  for (const std::string& line : split_lines(text))
    for (const std::string& t : split_ws(line)) vals.push_back(fortran_real(t));
  if ((int64_t)vals.size() < na)
    throw InputError("Error: File contains fewer values than expected (" +
                     std::to_string(vals.size()) + " out of " + std::to_string(na) + ").");
  if ((int64_t)vals.size() > na) throw InputError("Error: File contains more values than expected.");
  return vals;
}

std::string format_record(double time, const double* v, int64_t n) {
  char buf[48];
  std::snprintf(buf, sizeof(buf), "%15.8E", (double)(float)time);
  std::string out = " ";
  out += buf;
  for (int64_t i = 0; i < n; ++i) {
    std::snprintf(buf, sizeof(buf), " %24.16E", v[i]);
    out += buf;
  }
  out += "\n";
  return out;
}

std::string next_log_name(const std::string& outdir, const std::string& run_name) {
  const std::string rn = trim(run_name);
  for (int i = 0;; ++i) {
    char suffix[16];
    std::snprintf(suffix, sizeof(suffix), "_%02d", i);
    std::string name = outdir;
    if (!name.empty() && name.back() != '/') name += '/';
    name += "output_" + rn + suffix;
    struct stat st;
    if (stat(name.c_str(), &st) != 0) return name;
  }
}

std::vector<double> parse_property_table(const std::string& text, const std::string& name) {
  std::vector<double> rows;
  for (const std::string& line : split_lines(text)) {
    const std::vector<std::string> t = split_ws(line);
    if (t.empty()) continue;
    if (t.size() != 4)
      throw InputError("Error: " + name + ": each row needs 4 values (T, kappa, rho, c), got " +
                       std::to_string(t.size()));
    for (const std::string& v : t) rows.push_back(fortran_real(v));
    const size_t r = rows.size() / 4;
    if (r > 1 && !(rows[4 * (r - 1)] > rows[4 * (r - 2)]))
      throw InputError("Error: " + name + ": temperatures must ascend");
  }
  if (rows.size() < 8) throw InputError("Error: " + name + ": a table needs at least two rows");
  return rows;
}

PropertyTables load_material_tables(const std::string& inputs_dir, const System& sys) {
  PropertyTables pt;
  const int64_t n = sys.nx * sys.ny * sys.nz;
  std::map<int64_t, int32_t> index;              // material -> table, -1 without a file
  for (int64_t I = 0; I < n; ++I) index.emplace(sys.imaterial[I], -1);
  pt.offsets.push_back(0);
  for (auto& kv : index) {                       // ascending material index
    std::string path = inputs_dir;
    if (!path.empty() && path.back() != '/') path += '/';
    path += "MatTable" + std::to_string((long long)kv.first);
    struct stat st;
    if (stat(path.c_str(), &st) != 0) continue;  // no file: fixed properties
    const std::vector<double> rows =
        parse_property_table(read_text_file(path, "Error cannot find file: " + path), path);
    kv.second = pt.ntables();
    pt.materials.push_back(kv.first);
    pt.rows.insert(pt.rows.end(), rows.begin(), rows.end());
    pt.offsets.push_back((int32_t)(pt.rows.size() / 4));
  }
  pt.cell_table.resize(n);
  for (int64_t I = 0; I < n; ++I) pt.cell_table[I] = index[sys.imaterial[I]];
  return pt;
}

int records_after(const Param& p, int64_t itime) {
  if (p.test_run) return 0;
  int n = itime == 1 ? 1 : 0;
  if (p.write_to_txt && p.write_every > 0 && itime % p.write_every == 0) ++n;
  return n;
}

std::string problem_json(const Deck& d) {
  const Param& p = d.param;
  const hf_problem& q = d.prob;
  const int64_t n = d.ncells();
  std::ostringstream o;
  o << "{\"nx\": " << q.nx << ", \"ny\": " << q.ny << ", \"nz\": " << q.nz;
  o << ", \"lx\": " << json_num(q.lx) << ", \"ly\": " << json_num(q.ly) << ", \"lz\": " << json_num(q.lz);
  o << ", ";
  append_json_array(o, "kappa", d.kappa.data(), n);
  o << ", ";
  append_json_array(o, "rho", d.rho.data(), n);
  o << ", ";
  append_json_array(o, "heat_capacity", d.heat_capacity.data(), n);
  o << ", ";
  append_json_array(o, "tau", d.tau.data(), n);
  o << ", ";
  append_json_array(o, "em", d.em.data(), n);
  o << ", \"iheater\": [";
  for (int64_t i = 0; i < n; ++i) o << (i ? ", " : "") << d.sys.iheater[i];
  o << "], \"power_in\": " << json_num(q.power_in) << ", \"freq\": " << json_num(q.freq)
    << ", \"time_step\": " << json_num(q.time_step) << ", \"heated_steps\": " << q.heated_steps
    << ", \"icattaneo\": " << q.icattaneo << ", \"isteady\": " << q.isteady;
  o << ", \"periodic\": [" << q.periodic[0] << ", " << q.periodic[1] << ", " << q.periodic[2] << "]";
  o << ", \"cg_face\": [";
  for (int f = 0; f < 6; ++f) o << (f ? ", " : "") << q.cg_face[f];
  o << "], ";
  append_json_array(o, "kappa_bound", q.kappa_bound, 6);
  o << ", ";
  append_json_array(o, "t_bath_face", q.t_bath_face, 6);
  o << ", \"t_bath\": " << json_num(q.t_bath) << ", \"t_bath_cg\": " << json_num(q.t_bath_cg)
    << ", \"br\": " << json_num(q.br) << ", \"t_system\": " << json_num(p.t_system)
    << ", \"ntime\": " << p.ntime << ", \"write_every\": " << p.write_every
    << ", \"iverb\": " << p.iverb << ", \"run_name\": \"" << p.run_name << "\""
    << ", \"box\": [" << p.start_ix << ", " << p.end_ix << ", " << p.start_iy << ", " << p.end_iy
    << ", " << p.start_iz << ", " << p.end_iz << "]"
    << ", \"input_temp_dis\": " << (p.input_temp_dis ? 1 : 0)
    << ", \"full_restart\": " << (p.full_restart ? 1 : 0)
    << ", \"test_run\": " << (p.test_run ? 1 : 0)
    << ", \"write_to_txt\": " << (p.write_to_txt ? 1 : 0)
    << ", \"temp_dep_prop\": " << p.temp_dep_prop;
  if (d.tables.ntables() > 0) {
    const PropertyTables& t = d.tables;
    o << ", \"property_tables\": {\"materials\": [";
    for (size_t k = 0; k < t.materials.size(); ++k) o << (k ? ", " : "") << t.materials[k];
    o << "], \"offsets\": [";
    for (size_t k = 0; k < t.offsets.size(); ++k) o << (k ? ", " : "") << t.offsets[k];
    o << "], ";
    append_json_array(o, "rows", t.rows.data(), (int64_t)t.rows.size());
    o << ", \"cell_table\": [";
    for (size_t k = 0; k < t.cell_table.size(); ++k) o << (k ? ", " : "") << t.cell_table[k];
    o << "]}";
  }
  o << "}";
  return o.str();
}

}  // namespace hfhost
