// The reference's JSON run description read into cil_config / cil_colony_params, and its INIT
// built on the host (include/cil_input.h).
//
// Parser: a small recursive-descent JSON reader (RFC 8259 values; objects keep their key order
// and the last of repeated keys wins on lookup, as nlohmann::json's parse does). Accessors
// follow json_parser (JsonParser.hpp:13-135): a missing key, a wrong type, a value outside the
// accepted list or a vector of the wrong length is an error naming the key.
//
// INIT RANDOM (Input.cpp:736-757) draws, per cell, a uniform position in the box for every
// element, then for the front element a radius N(rss, 0.25 rss) and a direction angle
// uniform() * pi (3D also a second angle), and displaces the front element by that vector
// from its own uniform position, wrapped like Box::updatePos (Utils.hpp:556-565). rss is the
// two-element steady-state length sqrt(RMAX^2 (1 - alpha/beta KAPPA_PULL)),
// alpha = 1/zeta0 + 1/zeta1, beta = m0/zeta0 + m1/zeta1 (Input.cpp:139-144). initialize()
// reads INIT before and after initializeCellStatus (CIL.cuh:374-378), so a RANDOM start
// consumes the stream as positions, cell status, positions, and the second positions are kept.
// Cell status (CIL.cuh:253-330), dividing species only: per cell, unless CONST_FORCE, a
// uniform0x(1) test against p = tau_mig / (tau_mig + tau_div) picks the migration or division
// time span max(Nint(N(mu, sigma) / dt), 1) (randomTimeSpan, MD.cuh:434-436); then theta =
// uniform0x(1); then span -= Nint(uniform0x(span)) - 1 and tswitch = t0 + span with t0 = 0.
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <utility>
#include <vector>

#include "cil_cycle.h"
#include "cil_input.h"
#include "cil_h5.hpp"
#include "host_rng.h"

namespace {

// ---------------------------------------------------------------------------- JSON values
struct JVal {
  enum Kind { kNull, kBool, kNum, kStr, kArr, kObj } kind = kNull;
  bool b = false;
  double num = 0.0;
  std::string str;
  std::vector<JVal> arr;
  std::vector<std::pair<std::string, JVal>> obj;

  const JVal *find(const std::string &k) const {
    const JVal *hit = nullptr;
    for (const auto &kv : obj)
      if (kv.first == k) hit = &kv.second;
    return hit;
  }
};

const char *kind_name(JVal::Kind k) {
  switch (k) {
    case JVal::kNull: return "null";
    case JVal::kBool: return "boolean";
    case JVal::kNum: return "number";
    case JVal::kStr: return "string";
    case JVal::kArr: return "array";
    default: return "object";
  }
}

class Parser {
 public:
  explicit Parser(const std::string &s) : s_(s) {}

  JVal parse() {
    JVal v = value(0);
    ws();
    if (i_ != s_.size()) fail("trailing characters after the JSON value");
    return v;
  }

 private:
  [[noreturn]] void fail(const std::string &m) const {
    int line = 1;
    for (size_t k = 0; k < i_ && k < s_.size(); ++k) line += s_[k] == '\n';
    throw std::domain_error("JSON parse error at line " + std::to_string(line) + ": " + m);
  }
  void ws() {
    while (i_ < s_.size() && (s_[i_] == ' ' || s_[i_] == '\t' || s_[i_] == '\n' || s_[i_] == '\r')) ++i_;
  }
  bool eat(const char *lit) {
    const size_t n = strlen(lit);
    if (s_.compare(i_, n, lit) == 0) {
      i_ += n;
      return true;
    }
    return false;
  }
  JVal value(int depth) {
    if (depth > 256) fail("nesting too deep");
    ws();
    if (i_ >= s_.size()) fail("unexpected end of input");
    JVal v;
    const char c = s_[i_];
    if (c == '{') {
      v.kind = JVal::kObj;
      ++i_;
      ws();
      if (i_ < s_.size() && s_[i_] == '}') {
        ++i_;
        return v;
      }
      for (;;) {
        ws();
        if (i_ >= s_.size() || s_[i_] != '"') fail("expected a string key");
        std::string k = string();
        ws();
        if (i_ >= s_.size() || s_[i_] != ':') fail("expected ':' after key \"" + k + "\"");
        ++i_;
        v.obj.emplace_back(std::move(k), value(depth + 1));
        ws();
        if (i_ < s_.size() && s_[i_] == ',') {
          ++i_;
          continue;
        }
        if (i_ < s_.size() && s_[i_] == '}') {
          ++i_;
          return v;
        }
        fail("expected ',' or '}' in an object");
      }
    }
    if (c == '[') {
      v.kind = JVal::kArr;
      ++i_;
      ws();
      if (i_ < s_.size() && s_[i_] == ']') {
        ++i_;
        return v;
      }
      for (;;) {
        v.arr.push_back(value(depth + 1));
        ws();
        if (i_ < s_.size() && s_[i_] == ',') {
          ++i_;
          continue;
        }
        if (i_ < s_.size() && s_[i_] == ']') {
          ++i_;
          return v;
        }
        fail("expected ',' or ']' in an array");
      }
    }
    if (c == '"') {
      v.kind = JVal::kStr;
      v.str = string();
      return v;
    }
    if (eat("true")) {
      v.kind = JVal::kBool;
      v.b = true;
      return v;
    }
    if (eat("false")) {
      v.kind = JVal::kBool;
      return v;
    }
    if (eat("null")) return v;
    if (c == '-' || (c >= '0' && c <= '9')) {
      size_t j = i_;
      if (s_[j] == '-') ++j;
      const size_t digits = j;
      while (j < s_.size() && isdigit(static_cast<unsigned char>(s_[j]))) ++j;
      if (j == digits) fail("malformed number");
      if (j < s_.size() && s_[j] == '.') {
        ++j;
        const size_t f = j;
        while (j < s_.size() && isdigit(static_cast<unsigned char>(s_[j]))) ++j;
        if (j == f) fail("malformed number");
      }
      if (j < s_.size() && (s_[j] == 'e' || s_[j] == 'E')) {
        ++j;
        if (j < s_.size() && (s_[j] == '+' || s_[j] == '-')) ++j;
        const size_t e = j;
        while (j < s_.size() && isdigit(static_cast<unsigned char>(s_[j]))) ++j;
        if (j == e) fail("malformed number");
      }
      v.kind = JVal::kNum;
      v.num = std::strtod(s_.substr(i_, j - i_).c_str(), nullptr);
      i_ = j;
      return v;
    }
    fail(std::string("unexpected character '") + c + "'");
  }
  static void utf8(std::string &o, unsigned cp) {
    if (cp < 0x80) {
      o += static_cast<char>(cp);
    } else if (cp < 0x800) {
      o += static_cast<char>(0xC0 | (cp >> 6));
      o += static_cast<char>(0x80 | (cp & 0x3F));
    } else if (cp < 0x10000) {
      o += static_cast<char>(0xE0 | (cp >> 12));
      o += static_cast<char>(0x80 | ((cp >> 6) & 0x3F));
      o += static_cast<char>(0x80 | (cp & 0x3F));
    } else {
      o += static_cast<char>(0xF0 | (cp >> 18));
      o += static_cast<char>(0x80 | ((cp >> 12) & 0x3F));
      o += static_cast<char>(0x80 | ((cp >> 6) & 0x3F));
      o += static_cast<char>(0x80 | (cp & 0x3F));
    }
  }
  unsigned hex4() {
    if (i_ + 4 > s_.size()) fail("short \\u escape");
    unsigned v = 0;
    for (int k = 0; k < 4; ++k) {
      const char h = s_[i_++];
      v <<= 4;
      if (h >= '0' && h <= '9') v |= static_cast<unsigned>(h - '0');
      else if (h >= 'a' && h <= 'f') v |= static_cast<unsigned>(h - 'a' + 10);
      else if (h >= 'A' && h <= 'F') v |= static_cast<unsigned>(h - 'A' + 10);
      else fail("bad \\u escape");
    }
    return v;
  }
  std::string string() {
    ++i_;  // opening quote
    std::string o;
    for (;;) {
      if (i_ >= s_.size()) fail("unterminated string");
      const char c = s_[i_++];
      if (c == '"') return o;
      if (static_cast<unsigned char>(c) < 0x20) fail("control character in a string");
      if (c != '\\') {
        o += c;
        continue;
      }
      if (i_ >= s_.size()) fail("unterminated escape");
      const char e = s_[i_++];
      switch (e) {
        case '"': o += '"'; break;
        case '\\': o += '\\'; break;
        case '/': o += '/'; break;
        case 'b': o += '\b'; break;
        case 'f': o += '\f'; break;
        case 'n': o += '\n'; break;
        case 'r': o += '\r'; break;
        case 't': o += '\t'; break;
        case 'u': {
          unsigned cp = hex4();
          if (cp >= 0xD800 && cp < 0xDC00 && i_ + 1 < s_.size() && s_[i_] == '\\' && s_[i_ + 1] == 'u') {
            i_ += 2;
            const unsigned lo = hex4();
            if (lo >= 0xDC00 && lo < 0xE000) cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
          }
          utf8(o, cp);
          break;
        }
        default: fail(std::string("bad escape '\\") + e + "'");
      }
    }
  }

  const std::string &s_;
  size_t i_ = 0;
};

// ---------------------------------------------------------------------------- accessors
[[noreturn]] void key_error(const std::string &path, const std::string &m) {
  throw std::domain_error(path + " : " + m);
}

struct Node {
  const JVal *v;
  std::string path;

  bool has(const std::string &k) const { return v->kind == JVal::kObj && v->find(k) != nullptr; }
  Node child(const std::string &k) const {
    const std::string p = path.empty() ? k : path + "." + k;
    if (v->kind != JVal::kObj) key_error(p, std::string("parent is a ") + kind_name(v->kind) + ", not an object");
    const JVal *c = v->find(k);
    if (!c) key_error(p, "key not found");
    return Node{c, p};
  }
  double num(const std::string &k) const {
    Node c = child(k);
    if (c.v->kind != JVal::kNum) key_error(c.path, std::string("expected a number, got a ") + kind_name(c.v->kind));
    return c.v->num;
  }
  int integer(const std::string &k) const {
    const double d = num(k);
    if (d != std::floor(d) || std::fabs(d) > 2147483647.0) key_error(path + "." + k, "expected an integer");
    return static_cast<int>(d);
  }
  bool boolean(const std::string &k) const {
    Node c = child(k);
    if (c.v->kind != JVal::kBool) key_error(c.path, std::string("expected a boolean, got a ") + kind_name(c.v->kind));
    return c.v->b;
  }
  std::string str(const std::string &k) const {
    Node c = child(k);
    if (c.v->kind != JVal::kStr) key_error(c.path, std::string("expected a string, got a ") + kind_name(c.v->kind));
    return c.v->str;
  }
  std::string pick(const std::string &k, std::initializer_list<const char *> ok) const {
    const std::string s = str(k);
    std::string list;
    for (const char *o : ok) {
      if (s == o) return s;
      list += std::string(list.empty() ? "" : ", ") + o;
    }
    key_error(path + "." + k, "value " + s + " is not one of {" + list + "}");
  }
  const std::vector<JVal> &array(const std::string &k, Node *out = nullptr) const {
    Node c = child(k);
    if (c.v->kind != JVal::kArr) key_error(c.path, std::string("expected an array, got a ") + kind_name(c.v->kind));
    if (out) *out = c;
    return c.v->arr;
  }
  std::vector<double> nums(const std::string &k, size_t size) const {
    Node c{nullptr, ""};
    const auto &a = array(k, &c);
    if (a.size() != size)
      key_error(c.path, "vector should be of size " + std::to_string(size) + ". Got " + std::to_string(a.size()));
    std::vector<double> out;
    for (const auto &e : a) {
      if (e.kind != JVal::kNum) key_error(c.path, "expected numbers");
      out.push_back(e.num);
    }
    return out;
  }
  std::vector<bool> bools(const std::string &k, size_t size) const {
    Node c{nullptr, ""};
    const auto &a = array(k, &c);
    if (a.size() != size)
      key_error(c.path, "vector should be of size " + std::to_string(size) + ". Got " + std::to_string(a.size()));
    std::vector<bool> out;
    for (const auto &e : a) {
      if (e.kind != JVal::kBool) key_error(c.path, "expected booleans");
      out.push_back(e.b);
    }
    return out;
  }
  std::vector<std::string> strs(const std::string &k) const {
    Node c{nullptr, ""};
    const auto &a = array(k, &c);
    std::vector<std::string> out;
    for (const auto &e : a) {
      if (e.kind != JVal::kStr) key_error(c.path, "expected strings");
      out.push_back(e.str);
    }
    return out;
  }
  // [[a, b], ...]: pairs of strings (the DOMAIN SPECIES list, Input.cpp:318-322)
  std::vector<std::pair<std::string, std::string>> str_pairs(const std::string &k) const {
    Node c{nullptr, ""};
    const auto &a = array(k, &c);
    std::vector<std::pair<std::string, std::string>> out;
    for (const auto &e : a) {
      if (e.kind != JVal::kArr || e.arr.size() != 2) key_error(c.path, "Wrong cell pair specification");
      for (const auto &q : e.arr)
        if (q.kind != JVal::kStr) key_error(c.path, "expected strings");
      out.emplace_back(e.arr[0].str, e.arr[1].str);
    }
    return out;
  }
  // [[[cell, elem], [cell, elem]], ...]: pairs of (cell, element) names (the DOMAIN ELEMENTS
  // list, Input.cpp:330-345)
  std::vector<std::pair<std::pair<std::string, std::string>, std::pair<std::string, std::string>>> elem_pairs(
      const std::string &k) const {
    Node c{nullptr, ""};
    const auto &a = array(k, &c);
    std::vector<std::pair<std::pair<std::string, std::string>, std::pair<std::string, std::string>>> out;
    for (const auto &e : a) {
      if (e.kind != JVal::kArr || e.arr.size() != 2) key_error(c.path, "Wrong element pair specification");
      std::pair<std::string, std::string> ce[2];
      for (int q = 0; q < 2; ++q) {
        const JVal &x = e.arr[q];
        if (x.kind != JVal::kArr || x.arr.size() != 2 || x.arr[0].kind != JVal::kStr || x.arr[1].kind != JVal::kStr)
          key_error(c.path, "Wrong element pair specification");
        ce[q] = {x.arr[0].str, x.arr[1].str};
      }
      out.emplace_back(ce[0], ce[1]);
    }
    return out;
  }
};

constexpr double kPi = 3.14159265358979323846;  // M_PI, Constants::PI (Utils.hpp:42)

int nint(double a) { return a >= 0.0 ? static_cast<int>(a + 0.5) : static_cast<int>(a - 0.5); }  // Utils.hpp:172-174

void copy_str(char *dst, size_t cap, const std::string &s) {
  snprintf(dst, cap, "%s", s.c_str());
}

}  // namespace

// ---------------------------------------------------------------------------- the run
struct cil_input {
  std::string err;
  bool ok = false;
  JVal root;
  cil_config cfg{};
  cil_colony_params p{};
  cil_run_info run{};
  // species and INIT
  int dim = 2;
  double box[3] = {0, 0, 0};
  bool pbc[3] = {false, false, false};
  double dt = 0.0;
  double sigma[2] = {0, 0};
  double rss = 0.0;
  bool divide = false, const_force = false;
  double tau_div[2] = {0, 0}, tau_mig[2] = {0, 0};
  std::string init_kind;
  int ncells = 0;
  std::vector<double> json_pos;  // INIT JSON or H5: [cell][elements][dim]
  // INIT H5 ALL (Input.cpp:643-726): the cell status of the restart file
  bool h5_all = false;
  std::vector<double> h5_vel, h5_theta, h5_rho, h5_sigma;  // [cell][elem][dim], [cell], [cell], [cell][elem]
  std::vector<int> h5_state;
  // MD keys of either model
  bool drain = false;
  double osm = 0.0;
  double dpd_same = 0.0, dpd_diff = 0.0, dpd_bg = 0.0, kbt = 0.0;  // MD.INTEGRATOR.DPD, MD.KBT
  // single-element species: the cell-cycle model (cil_cycle.h)
  int nelem = 2;
  cil_cycle_params cyc{};
};

namespace {

// INIT H5 (Input.cpp:610-726): LOCATION [file, dataset] reads the element positions; ALL [file,
// R, Vel, State, Theta, RHO, SigmaCore] the cell status too. RANGE [first, end) selects cells
// (negative values count from the end). The file is opened as given, relative to the working
// directory, as the reference opens it.
void read_h5_init(cil_input *in, const Node &h, int nelem) {
  const std::string how = h.pick("SELECT", {"ALL", "LOCATION"});
  const bool all = how == "ALL";
  const auto names = h.strs(how);
  if (names.size() != (all ? 7u : 2u))
    key_error(h.path + "." + how, "vector should be of size " + std::to_string(all ? 7 : 2) + ". Got " +
                                      std::to_string(names.size()));
  cil::h5::Reader r;
  std::string err;
  if (!r.open(names[0], &err)) key_error(h.path + "." + how, err);
  auto load = [&](const std::string &ds_name, std::vector<double> *out, uint64_t per_cell) -> uint64_t {
    cil::h5::Dataset ds;
    if (!r.dataset(ds_name, &ds, &err) || !r.read(ds, out, &err)) key_error(h.path + "." + how, err);
    if (per_cell == 0 || out->size() % per_cell) key_error(h.path + "." + how, "Inconsistent H5 dataset dimensions");
    return out->size() / per_cell;
  };
  const uint64_t D = static_cast<uint64_t>(in->dim), E = static_cast<uint64_t>(nelem);
  std::vector<double> pos;
  const long long ncells = static_cast<long long>(load(names[1], &pos, E * D));
  long long lo = 0, hi = ncells;
  if (h.has("RANGE")) {
    const auto rg = h.nums("RANGE", 2);
    lo = static_cast<long long>(rg[0]);
    hi = static_cast<long long>(rg[1]);
    if (lo < 0) lo += ncells;
    if (hi < 0) hi += ncells;
  }
  if (lo < 0 || lo > ncells || hi < 0 || hi > ncells) key_error(h.path + ".RANGE", "Range out of bounds");
  if (!(lo < hi)) key_error(h.path + ".RANGE", "Range is empty");
  in->ncells = static_cast<int>(hi - lo);
  in->json_pos.assign(pos.begin() + lo * E * D, pos.begin() + hi * E * D);
  if (!all) return;
  in->h5_all = true;
  std::vector<double> vel, state, theta, rho, sigma;
  auto same = [&](uint64_t n, const char *what) {
    if (static_cast<long long>(n) != ncells)
      key_error(h.path + ".ALL", std::string(what) + ": Inconsistent H5 dataset dimensions");
  };
  same(load(names[2], &vel, E * D), "Vel");
  same(load(names[3], &state, 1), "State");
  same(load(names[4], &theta, 1), "Theta");
  same(load(names[5], &rho, 1), "RHO");
  same(load(names[6], &sigma, E), "SigmaCore");
  in->h5_vel.assign(vel.begin() + lo * E * D, vel.begin() + hi * E * D);
  in->h5_theta.assign(theta.begin() + lo, theta.begin() + hi);
  in->h5_rho.assign(rho.begin() + lo, rho.begin() + hi);
  in->h5_sigma.assign(sigma.begin() + lo * E, sigma.begin() + hi * E);
  in->h5_state.clear();
  for (long long i = lo; i < hi; ++i) in->h5_state.push_back(static_cast<int>(state[i]));
}

// INIT block of either model: RANDOM cell count, or JSON element positions (rows of DIM)
void read_init(cil_input *in, const Node &root, const std::string &cell, int nelem) {
  Node init = root.child("INIT").child(cell);
  in->init_kind = init.pick("SELECT", {"JSON", "H5", "RANDOM"});
  if (in->init_kind == "H5") {
    read_h5_init(in, init.child("H5"), nelem);
    return;
  }
  if (in->init_kind == "RANDOM") {
    const int n = init.child("RANDOM").integer("NUMBER");
    if (n < 0) key_error(init.path + ".RANDOM.NUMBER", "negative cell count");
    in->ncells = n;
    return;
  }
  Node jn{nullptr, ""};
  const auto &rows = init.array("JSON", &jn);
  if (rows.size() % nelem) key_error(jn.path, "element count is not a multiple of NELEM");
  in->ncells = static_cast<int>(rows.size() / nelem);
  in->json_pos.reserve(rows.size() * in->dim);
  for (const auto &r : rows) {
    if (r.kind != JVal::kArr || r.arr.size() != static_cast<size_t>(in->dim))
      key_error(jn.path, "rows should be of size " + std::to_string(in->dim));
    for (const auto &x : r.arr) {
      if (x.kind != JVal::kNum) key_error(jn.path, "expected numbers");
      in->json_pos.push_back(x.num);
    }
  }
}

// A single-element species: the cell-cycle model (readSpecs, Input.cpp:6-262, for NELEM 1)
void read_single(cil_input *in, const Node &root, const Node &loc, const std::string &cell,
                 const std::string &integrator, const std::string &pair) {
  in->nelem = 1;
  cil_cycle_params &q = in->cyc;
  cil_run_info &run = in->run;
  const auto enames = loc.strs("NAMES");
  if (enames.size() != 1) key_error(loc.path + ".NAMES", "vector should be of size 1. Got " + std::to_string(enames.size()));
  copy_str(run.elem_names[0], sizeof run.elem_names[0], enames[0]);
  run.elem_names[1][0] = 0;
  if (integrator == "STOCHASTIC_HEUN")
    key_error("MD.INTEGRATOR.SELECT", "the single-element model runs EULER or STOCHASTIC_EULER");
  if (pair != "HZ") key_error("INTERACTIONS.PAIRFORCES.SELECT", "the single-element model's contacts are the Hertz law (HZ)");
  q.dim = in->dim;
  for (int d = 0; d < 3; ++d) {
    q.box[d] = in->box[d];
    q.periodic[d] = in->pbc[d] ? 1 : 0;
  }
  q.dt = in->dt;
  Node hz = loc.child("PAIRFORCES").child("HZ");
  q.E = hz.nums("ELASTIC_MODULUS", 1)[0];
  q.nu = hz.nums("POISSON_RATIO", 1)[0];
  q.sigma_core = hz.nums("SIGMA_CORE", 1)[0];
  q.adhesion = hz.nums("ADHESION_CONSTANT", 1)[0];
  q.motility = loc.nums("MOTILITY", 1)[0];
  q.zeta = loc.nums("FRICTION", 1)[0];
  const bool dpd = integrator == "DPD";
  if (!dpd && !(q.zeta > 0.0)) key_error(loc.path + ".FRICTION", "In Euler, zeta should > 0!!!");
  q.zeta_p = loc.nums("P_FRICTION", 1)[0];
  q.zeta_p_beta = loc.nums("P_FRICTION_BETA", 1)[0];
  // NOISE_ON only with the stochastic integrators (Input.cpp:527-535)
  q.noise_D = (integrator == "EULER" || dpd) ? 0.0 : loc.child("NOISE").num("PASSIVE");
  q.integrator = dpd ? CIL_CYCLE_DPD : CIL_CYCLE_EULER;
  if (dpd) {
    q.mass = loc.nums("MASS", 1)[0];
    if (!(q.mass > 0.0)) key_error(loc.path + ".MASS", "DPD needs a positive mass");
    q.kbt = in->kbt;
    q.dis_same = in->dpd_same;
    q.dis_diff = in->dpd_diff;
    q.dis_bg = in->dpd_bg;
  }
  q.osmotic_pressure = in->osm;
  q.drain = in->drain ? 1 : 0;
  q.cycle_rho_ratio = 1.0;  // Cell.cuh:242-254 defaults
  q.cycle_r_maxed = 1.0;
  q.v1 = 1.0;
  Node dv = loc.child("DIVISION");
  q.divide = dv.boolean("ENABLED") ? 1 : 0;
  if (q.divide) {
    if (dv.boolean("CONST_FORCE"))
      key_error(dv.path + ".CONST_FORCE", "constant-force cells do not enter the single-element cycle");
    q.tau_div_mu = dv.child("TAU_DIVISION").num("AVG");
    q.tau_div_sigma = dv.child("TAU_DIVISION").num("SIGMA");
    q.tau_mig_mu = dv.child("TAU_MIGRATION").num("AVG");
    q.tau_mig_sigma = dv.child("TAU_MIGRATION").num("SIGMA");
    if (q.tau_mig_mu != 0.0)
      key_error(dv.path + ".TAU_MIGRATION.AVG", "crawling cells never re-enter the single-element cycle (must be 0)");
    q.v1 = dv.num("V1");
    q.cycle_tau_r = dv.num("CYCLE_TAU_R");
    q.cycle_tau_v = dv.num("CYCLE_TAU_V");
    q.cycle_tau_p = dv.num("CYCLE_TAU_P");
    q.cycle_sigma_min = dv.num("CYCLE_SIGMA_MIN");
    q.cycle_p0 = dv.num("CYCLE_P0");
    q.cycle_beta_vs = dv.num("CYCLE_BETA_VS");
    q.cycle_rho_ratio = dv.num("CYCLE_RHO_RATIO");
    if (dv.has("CYCLE_R_MAXED")) q.cycle_r_maxed = dv.num("CYCLE_R_MAXED");
    if (dv.has("CYCLE_P_SHIFT")) q.cycle_p_shift = dv.num("CYCLE_P_SHIFT");
    if (dv.has("CYCLE_P_SHIFT_TAU")) q.cycle_p_shift_tau = dv.num("CYCLE_P_SHIFT_TAU");
  }
  if (loc.has("APOPTOSIS") && loc.child("APOPTOSIS").boolean("ENABLED")) {  // Input.cpp:247-262
    Node a = loc.child("APOPTOSIS");
    // the law each step applies: Euler calculApoptosisCyclePressure (CIL.cu:1017), DPD
    // calculApoptosisPressureTime (CIL.cu:1064)
    q.apoptosis = dpd ? CIL_APOP_PRESSURE_TIME : CIL_APOP_CYCLE_PRESSURE;
    q.apop_pressure = a.num("APOP_PRESSURE");
    q.apop_duration = a.num("APOP_DURATION");
    q.apop_rate = a.num("APOP_RATE");
    q.extr_gamma = a.num("EXTR_GAMMA");
    (void)a.num("APOP_ACTIVITY_ALPHA");
    (void)a.num("APOP_GAMMA");
    q.extr_rate = a.num("EXTR_RATE");
    if (!(q.apop_rate * q.dt < 1.0)) key_error(a.path + ".APOP_RATE", "Apoptosis rate per time step >= 1");
  }
  const bool has_gpu = root.has("GPU");
  // GPU.PRECISION: FP64 (the default here: the reference's arithmetic) or MIXED (FP32 pair terms)
  if (has_gpu && root.child("GPU").has("PRECISION"))
    q.precision = root.child("GPU").pick("PRECISION", {"FP64", "MIXED"}) == "MIXED" ? 1 : 0;
  read_init(in, root, cell, 1);
  run.ncells = in->ncells;
  run.capacity = has_gpu && root.child("GPU").has("CAPACITY") ? root.child("GPU").integer("CAPACITY")
                                                                : 4 * in->ncells + 64;
}

void read_all(cil_input *in) {
  Node root{&in->root, ""};
  if (in->root.kind != JVal::kObj) throw std::domain_error("the run description must be a JSON object");
  {  // units (CIL.cuh:340-342): the Units class is not in the reference tree
    Node u = root.child("UNITS");
    for (const char *k : {"LENGTH", "MOTILITY", "FRICTION"})
      if (u.num(k) != 1.0)
        key_error(u.path + "." + k, "unit scales other than 1 need the reference's Units class, which is not in its tree");
  }
  cil_config &cfg = in->cfg;
  cil_colony_params &p = in->p;
  cil_run_info &run = in->run;
  std::string integrator;
  {  // readMD (Input.cpp:501-558)
    Node md = root.child("MD");
    in->dim = md.integer("DIM");
    if (in->dim != 2 && in->dim != 3) key_error("MD.DIM", "value must be 2 or 3");
    run.gts = nint(md.num("GTS"));
    run.frames = nint(md.num("FRAMES"));
    const auto L = md.nums("BOX", in->dim);
    const auto pbc = md.bools("PBC", in->dim);
    for (int d = 0; d < in->dim; ++d) {
      in->box[d] = L[d];
      in->pbc[d] = pbc[d];
      if (!(L[d] > 0.0)) key_error("MD.BOX", "box lengths must be positive");
    }
    integrator = md.child("INTEGRATOR").pick("SELECT", {"EULER", "STOCHASTIC_EULER", "STOCHASTIC_HEUN", "DPD"});
    if (integrator == "DPD") {  // Input.cpp:538-544, 555-556 (units all 1)
      Node dpd = md.child("INTEGRATOR").child("DPD");
      in->dpd_same = dpd.num("DISSAMCEL");
      in->dpd_diff = dpd.num("DISDIFCEL");
      in->dpd_bg = dpd.num("DISBG");
      in->kbt = md.num("KBT");
    }
    Node dtn = md.child("DT");  // initializeTimeStep (CIL.cuh:167-250)
    if (dtn.pick("SELECT", {"AUTOSCALE", "MANUAL"}) == "AUTOSCALE")
      key_error("MD.DT.SELECT", "AUTOSCALE needs the reference's force-law time scales; use MANUAL");
    in->dt = dtn.num("MANUAL");
    if (!(in->dt > 0.0)) key_error("MD.DT.MANUAL", "dt <= 0");
    in->drain = md.boolean("DRAIN");
    in->osm = md.num("OSMOTIC_PRESSURE");
  }
  std::string pair = root.child("INTERACTIONS").child("PAIRFORCES").pick("SELECT", {"LJ", "SC", "HZ", "EA", "GHOSTS"});
  {  // readRunTime (Input.cpp:560-588)
    const int seed = root.child("RUNTIME").child("RNG").integer("SEED");
    run.seed = seed > 0 ? seed : static_cast<int>(time(nullptr));
  }
  {  // readOutput (Input.cpp:763-800)
    Node out = root.child("OUTPUT");
    copy_str(run.output_dir, sizeof run.output_dir, out.str("DIR"));
    copy_str(run.output_name, sizeof run.output_name, out.str("NAME"));
    for (const auto &f : out.strs("FORMAT")) {
      if (f == "GSD") run.output_gsd = 1;
      if (f == "H5") run.output_h5 = 1;
    }
  }
  // readSpecs (Input.cpp:6-300): one species of two-element cells
  Node sp = root.child("SPECIES");
  const auto names = sp.strs("DEFINE");
  if (names.size() != 1)
    key_error("SPECIES.DEFINE", "the GPU step runs one species per colony (got " + std::to_string(names.size()) + ")");
  const std::string cell = names[0];
  copy_str(run.cell_name, sizeof run.cell_name, cell);
  Node loc = sp.child(cell);
  const int nelem = loc.integer("NELEM");
  if (nelem == 1) {
    read_single(in, root, loc, cell, integrator, pair);
    return;
  }
  if (nelem != 2) key_error(loc.path + ".NELEM", "the GPU step models cells of one or two elements");
  if (integrator == "DPD")  // its step divides with calculDivisionsSingle (CIL.cu:1063)
    key_error("MD.INTEGRATOR.SELECT", "the GPU step runs DPD for single-element cells (NELEM 1)");
  const auto enames = loc.strs("NAMES");
  if (enames.size() != 2) key_error(loc.path + ".NAMES", "vector should be of size 2. Got " + std::to_string(enames.size()));
  if (enames[0] == enames[1]) key_error(loc.path + ".NAMES", "element names must be unique!");
  copy_str(run.elem_names[0], sizeof run.elem_names[0], enames[0]);
  copy_str(run.elem_names[1], sizeof run.elem_names[1], enames[1]);
  const auto m = loc.nums("MOTILITY", 2);
  const auto zeta = loc.nums("FRICTION", 2);
  for (int j = 0; j < 2; ++j)
    if (!(zeta[j] > 0.0)) key_error(loc.path + ".FRICTION", "In Euler, zeta should > 0!!!");
  Node pf = loc.child("PAIRFORCES");
  std::vector<double> eps_lj;
  if (pair == "LJ") {
    Node lj = pf.child("LJ");
    const auto s = lj.nums("SIGMA", 2);
    in->sigma[0] = s[0];
    in->sigma[1] = s[1];
    eps_lj = lj.nums("EPSILON", 2);
  } else if (pair == "SC") {
    const auto s = pf.child("SC").nums("SIGMA_CORE", 2);
    in->sigma[0] = s[0];
    in->sigma[1] = s[1];
  } else if (pair == "HZ" || pair == "EA") {
    const auto s = pf.child("HZ").nums("SIGMA_CORE", 2);
    in->sigma[0] = s[0];
    in->sigma[1] = s[1];
  } else {
    key_error("INTERACTIONS.PAIRFORCES.SELECT", "GHOSTS is not modelled by the GPU step");
  }
  double noise_D = 0.0, noise_r = 0.0, noise_a = 0.0;
  std::string noise_path;
  if (integrator != "EULER") {  // NOISE_ON (Input.cpp:527-535, 99-111)
    Node nz = loc.child("NOISE");
    noise_D = nz.num("PASSIVE");
    noise_path = nz.path;
    if (integrator == "STOCHASTIC_HEUN") {  // NOISE_ACTIVE: radial and angular noise of the cell axis
      noise_r = nz.num("RADIAL");
      noise_a = nz.num("ANGULAR");
      if ((noise_r != 0.0 || noise_a != 0.0) && in->dim == 3)
        key_error("MD.INTEGRATOR.SELECT", "Active noise not yet implemented for 3D systems");
    }
  }
  {  // steady-state length (Input.cpp:139-144) for INIT RANDOM
    Node fene = loc.child("FENE");
    const double kappa = fene.nums("KAPPA_PULL", 1)[0];
    const double rmax = fene.nums("RMAX", 1)[0];
    const double alpha = 1.0 / zeta[0] + 1.0 / zeta[1];
    const double beta = m[0] * (1.0 / zeta[0]) + m[1] * (1.0 / zeta[1]);
    in->rss = std::sqrt(rmax * rmax * (1.0 - alpha / beta * kappa));
  }
  {  // division (Input.cpp:148-245)
    Node dv = loc.child("DIVISION");
    in->divide = dv.boolean("ENABLED");
    if (in->divide) {
      in->const_force = dv.boolean("CONST_FORCE");
      in->tau_div[0] = dv.child("TAU_DIVISION").num("AVG");
      in->tau_div[1] = dv.child("TAU_DIVISION").num("SIGMA");
      in->tau_mig[0] = dv.child("TAU_MIGRATION").num("AVG");
      in->tau_mig[1] = dv.child("TAU_MIGRATION").num("SIGMA");
    }
  }
  double apop = 0.0;
  if (loc.has("APOPTOSIS") && loc.child("APOPTOSIS").boolean("ENABLED")) {  // Input.cpp:247-262
    apop = loc.child("APOPTOSIS").num("APOP_RATE");
    if (!(apop * in->dt < 1.0)) key_error(loc.path + ".APOPTOSIS.APOP_RATE", "Apoptosis rate per time step >= 1");
  }

  // the library's own block
  const bool has_gpu = root.has("GPU");
  Node gpu = has_gpu ? root.child("GPU") : Node{nullptr, "GPU"};
  auto gnum = [&](const char *k, double dflt) { return has_gpu && gpu.has(k) ? gpu.num(k) : dflt; };
  auto gpick = [&](const char *k, std::initializer_list<const char *> ok, const char *dflt) {
    return has_gpu && gpu.has(k) ? gpu.pick(k, ok) : std::string(dflt);
  };
  cfg.dim = in->dim;
  cfg.integrator = integrator == "STOCHASTIC_HEUN" ? CIL_INTEGRATOR_HEUN : CIL_INTEGRATOR_EULER;
  cfg.precision = gpick("PRECISION", {"FP64", "MIXED"}, "MIXED") == "FP64" ? CIL_PREC_FP64 : CIL_PREC_MIXED;
  cfg.rng_mode = gpick("RNG", {"PHILOX", "DSFMT"}, "PHILOX") == "DSFMT" ? CIL_RNG_DSFMT : CIL_RNG_PHILOX;
  cfg.seed = static_cast<uint64_t>(static_cast<uint32_t>(run.seed));
  cfg.num_colonies = 1;
  cfg.skin = cfg.precision == CIL_PREC_MIXED ? gnum("SKIN", 0.3) : 0.0;
  run.use_scheduler = has_gpu && gpu.has("SCHEDULER") ? gpu.boolean("SCHEDULER") : 0;
  const bool law_given = has_gpu && gpu.has("FORCE_LAW");
  if (law_given) {
    const std::string law = gpu.pick("FORCE_LAW", {"LJ_WCA", "SOFTCORE", "HERTZ"});
    cfg.force_law = law == "LJ_WCA" ? CIL_FORCE_LJ_WCA : law == "SOFTCORE" ? CIL_FORCE_SOFTCORE : CIL_FORCE_HERTZ;
    p.epsilon = gpu.num("EPSILON");
    p.rcut_scale = gnum("RCUT_SCALE", law == "LJ_WCA" ? std::pow(2.0, 1.0 / 6.0) : 1.0);
  } else if (pair == "LJ") {
    // readInteractionsLJ (Input.cpp:294-352): the WCA cutoff rc2 = 2^(1/3), or with ATTRACTION ON
    // rc2 = RCUT^2 over the pairs its DOMAIN names and SHIFT FORCE -> OPT::FORCE_SHIFTED
    Node att = root.child("INTERACTIONS").child("PAIRFORCES").child("LJ").child("ATTRACTION");
    if (eps_lj[0] != eps_lj[1])
      key_error(loc.path + ".PAIRFORCES.LJ.EPSILON", "the GPU step uses one epsilon per species");
    cfg.force_law = CIL_FORCE_LJ_WCA;
    p.epsilon = eps_lj[0];
    p.rcut_scale = std::pow(2.0, 1.0 / 6.0);
    p.force_shifted = 0;
    if (att.pick("SELECT", {"ON", "OFF"}) == "ON") {
      Node on = att.child("ON");
      const double rcut = on.num("RCUT");
      if (on.pick("SHIFT", {"FORCE", "POTENTIAL"}) == "FORCE") p.force_shifted = 1;
      if (!(rcut * rcut >= std::pow(2.0, 1.0 / 3.0))) key_error(on.path + ".RCUT", "Invalid LJ cutoff");
      Node dom = on.child("DOMAIN");
      const std::string sel = dom.pick("SELECT", {"ALL", "SPECIES", "ELEMENTS"});
      // one species of two elements: the domain covers all three element pairs or none of them
      int covered = 0;
      if (sel == "ALL") {
        covered = 3;
      } else if (sel == "SPECIES") {
        for (const auto &pr : dom.str_pairs("SPECIES")) {
          if (pr.first != cell || pr.second != cell)
            key_error(dom.path + ".SPECIES", "unknown cell type in " + pr.first + ", " + pr.second);
          covered = 3;
        }
      } else {
        bool pairs[2][2] = {{false, false}, {false, false}};
        for (const auto &pr : dom.elem_pairs("ELEMENTS")) {
          int e[2];
          for (int k = 0; k < 2; ++k) {
            const auto &ce = k == 0 ? pr.first : pr.second;
            if (ce.first != cell) key_error(dom.path + ".ELEMENTS", "Unknown cell type " + ce.first);
            if (ce.second == enames[0]) {
              e[k] = 0;
            } else if (ce.second == enames[1]) {
              e[k] = 1;
            } else {
              key_error(dom.path + ".ELEMENTS", "Unknown element name " + ce.second + " for cell type " + ce.first);
            }
          }
          pairs[e[0]][e[1]] = pairs[e[1]][e[0]] = true;
        }
        covered = (pairs[0][0] ? 1 : 0) + (pairs[0][1] ? 1 : 0) + (pairs[1][1] ? 1 : 0);
      }
      if (covered == 3) {
        p.rcut_scale = rcut;
      } else if (covered != 0) {
        key_error(dom.path + ".ELEMENTS", "the GPU step uses one cutoff per species (the attraction must cover "
                                          "all element pairs of the cell or none)");
      }
    }
  } else if (pair == "SC") {
    // the cubic well of SCParams (MD.cuh:134-232) with the element values of Input.cpp:48-62
    // (xi = SIGMA_RATIO * SIGMA_CORE, Em = EPSILON_RATIO * EPSILON_CORE) and rc2 = 1
    // (Input.cpp:354-357); MD.cu:57-75 averages the per-element values into per-pair ones,
    // which the GPU step holds as one value per colony, so the two elements must agree.
    Node sc = pf.child("SC");
    const auto e0 = sc.nums("EPSILON_CORE", 2);
    const auto sr = sc.nums("SIGMA_RATIO", 2);
    const auto er = sc.nums("EPSILON_RATIO", 2);
    for (int j = 0; j < 2; ++j)
      if (!(sr[j] <= 1.0)) key_error(sc.path + ".SIGMA_RATIO", "Sigma Ratio > 1 !!!");
    const double xi0 = sr[0] * in->sigma[0], xi1 = sr[1] * in->sigma[1];
    if (e0[0] != e0[1]) key_error(sc.path + ".EPSILON_CORE", "the GPU step uses one core energy per species");
    if (xi0 != xi1)
      key_error(sc.path + ".SIGMA_RATIO", "the GPU step uses one well width per species (SIGMA_RATIO x SIGMA_CORE "
                                          "equal for both elements)");
    if (er[0] * e0[0] != er[1] * e0[1])
      key_error(sc.path + ".EPSILON_RATIO", "the GPU step uses one well depth per species");
    cfg.force_law = CIL_FORCE_SC;
    p.epsilon = e0[0];
    p.well_epsilon = er[0] * e0[0];
    p.well_sigma = xi0;
    p.rcut_scale = 1.0;
    p.force_shifted = 0;  // FORCE_SHIFTED is set only by the LJ attraction block (Input.cpp:306)
  } else {
    // HZ: cellCellForce (MD.cu:757-790) calls the overload of HZParams::elemForce that passes
    // zero diameters (MD.cuh:265-270), so its force is -0 for every pair; EA: -Ei r^2 on every
    // link-list candidate (MD.cuh:297-304, 317-322), so it depends on the bin size
    key_error("GPU.FORCE_LAW", "the reference's two-element " + pair +
                                   (pair == "HZ" ? " force is zero for every pair (HZParams::elemForce with zero "
                                                   "diameters)"
                                                 : " force acts on every link-list candidate (bin-size dependent)") +
                                   "; set GPU.FORCE_LAW, EPSILON (and RCUT_SCALE)");
  }
  if (has_gpu && gpu.has("SPRING")) {  // the linear spring with the rest length growing over the cycle
    for (const auto &kv : {std::make_pair("RADIAL", noise_r), std::make_pair("ANGULAR", noise_a)})
      if (kv.second != 0.0)
        key_error(noise_path + "." + kv.first, "the active noise acts on the reference's bond (no GPU.SPRING)");
    Node spring = gpu.child("SPRING");
    p.kappa = spring.num("KAPPA");
    p.rest0 = spring.num("REST0");
    p.rest1 = spring.has("REST1") ? spring.num("REST1") : p.rest0;
  } else {
    // the reference's own bond (binaryCellForce, MD.cu:525-598) from the species' FENE block
    // (Input.cpp:115-136) and its CIL flag (Input.cpp:22); dividing cells run the reference's
    // crawling/dividing states (calculDivisions, CIL.cu:369-455) with the DIVISION block's R0,
    // Rmin, Rmin_RATIO and TAU_MIGRATION, the species' GROWTHK0/1/2 (Input.cpp:36-38, 153-243)
    Node fene = loc.child("FENE");
    if (in->divide) {
      Node dv = loc.child("DIVISION");
      p.div_r0 = dv.num("R0");
      p.div_rmin = dv.num("Rmin");
      p.div_rmin_ratio = dv.num("Rmin_RATIO");
      p.mig_tau_mu = in->tau_mig[0];
      p.mig_tau_sigma = in->tau_mig[1];
      const auto k0 = loc.nums("GROWTHK0", 2), k1 = loc.nums("GROWTHK1", 2), k2 = loc.nums("GROWTHK2", 2);
      for (int j = 0; j < 2; ++j) {
        p.growth_k0[j] = k0[j];
        p.growth_k1[j] = k1[j];
        p.growth_k2[j] = k2[j];
        p.sigma_core[j] = in->sigma[j];
      }
      p.fene_rmax_division = fene.has("RMAX_DIVISION") ? fene.nums("RMAX_DIVISION", 1)[0] : 0.0;
      p.div_swelling = dv.has("SWELLING") && dv.boolean("SWELLING") ? 1 : 0;
      // bins rebuilt every step; the reference's own draws unless GPU.RNG asks for the device's
      cfg.skin = 0.0;
      if (!(has_gpu && gpu.has("RNG"))) cfg.rng_mode = CIL_RNG_DSFMT;
    }
    p.intra_law = CIL_INTRA_FENE;
    p.cil = loc.boolean("CIL") ? 1 : 0;
    p.fene_kappa = fene.nums("KAPPA_PULL", 1)[0];
    p.fene_kappa_push = fene.nums("KAPPA_PUSH", 1)[0];
    p.fene_spring_ratio = fene.nums("SPRING_RATIO", 1)[0];
    p.fene_rmax = fene.nums("RMAX", 1)[0];
    if (!(p.fene_spring_ratio >= 0.0 && p.fene_spring_ratio < 1.0))
      key_error(fene.path + ".SPRING_RATIO", "the GPU step needs 0 <= SPRING_RATIO < 1");
    if (noise_r != 0.0 || noise_a != 0.0) {
      // the bond's active noise (CIL.cu:803-815, MD.cu:573-579): drawn with the reference's stream
      p.noise_radial = noise_r;
      p.noise_angular = noise_a;
      cfg.rng_mode = CIL_RNG_DSFMT;
      cfg.skin = 0.0;
      if (has_gpu && gpu.has("RNG") && gpu.pick("RNG", {"PHILOX", "DSFMT"}) != "DSFMT")
        key_error("GPU.RNG", "the bond's active noise runs with the reference's draws (DSFMT)");
    }
  }
  p.noise_per_cell = has_gpu && gpu.has("NOISE_PER_CELL") ? gpu.boolean("NOISE_PER_CELL") : 0;
  if (has_gpu && gpu.has("WALLS")) {
    Node w = gpu.child("WALLS");
    const auto pos = w.nums("POS", w.array("POS").size());
    const auto dir = w.nums("DIR", pos.size());
    if (pos.size() > 2) key_error(w.path + ".POS", "at most two walls");
    p.nwalls = static_cast<int32_t>(pos.size());
    for (size_t k = 0; k < pos.size(); ++k) {
      p.wall_pos[k] = pos[k];
      p.wall_dir[k] = dir[k] > 0 ? 1 : -1;
    }
    p.wall_E = w.num("E");
  }
  p.dim = in->dim;
  p.force_law = cfg.force_law;
  p.divide = in->divide ? 1 : 0;
  for (int d = 0; d < 3; ++d) {
    p.box[d] = in->box[d];
    p.periodic[d] = in->pbc[d] ? 1 : 0;
  }
  p.zeta[0] = zeta[0];
  p.zeta[1] = zeta[1];
  p.motility[0] = m[0];
  p.motility[1] = m[1];
  p.noise_D = noise_D;
  p.dt = in->dt;
  p.div_tau_mu = in->tau_div[0];
  p.div_tau_sigma = in->tau_div[1];
  p.apop_rate = apop;

  read_init(in, root, cell, 2);  // readInit (Input.cpp:591-761)
  run.ncells = in->ncells;
  run.capacity = has_gpu && gpu.has("CAPACITY") ? gpu.integer("CAPACITY") : 4 * in->ncells + 64;
}

// INIT RANDOM positions of every cell (Input.cpp:736-757).
void random_positions(cil::HostRng &rng, const cil_input *in, double *pos) {
  const int D = in->dim;
  for (int i = 0; i < in->ncells; ++i) {
    double *R = pos + static_cast<size_t>(i) * 2 * D;
    for (int j = 0; j < 2; ++j)
      for (int d = 0; d < D; ++d) R[j * D + d] = rng.uniform0x(in->box[d]);
    const double radius = rng.normal(in->rss, 0.25 * in->rss);
    const double theta = rng.uniform() * kPi;
    const double sinphi = D == 2 ? 1.0 : rng.uniform() * kPi;
    const double dir[3] = {sinphi * std::cos(theta), sinphi * std::sin(theta), std::sqrt(1.0 - sinphi * sinphi)};
    for (int d = 0; d < D; ++d) {  // Box::updatePos(r, v, dt) (Utils.hpp:561-565)
      double &r = R[D + d];
      r = in->pbc[d] ? std::fmod(r + radius * dir[d] + in->box[d], in->box[d]) : r + dir[d] * radius;
    }
  }
}

int time_span(cil::HostRng &rng, const double tau[2], double dt) {  // randomTimeSpan (MD.cuh:434-436)
  const int s = nint(rng.normal(tau[0], tau[1]) / dt);
  return s > 1 ? s : 1;
}

}  // namespace

extern "C" {

cil_status cil_input_load(const char *text, int32_t is_path, cil_input **out) {
  if (!text) return CIL_ERR_CONFIG;
  cil_input *in = new cil_input();
  if (out) *out = in;
  try {
    std::string doc;
    if (is_path) {
      std::ifstream f(text, std::ios::binary);
      if (!f) {
        in->err = std::string(text) + ": cannot open (" + strerror(errno) + ")";
        if (!out) delete in;
        return CIL_ERR_IO;
      }
      std::ostringstream ss;
      ss << f.rdbuf();
      doc = ss.str();
    } else {
      doc = text;
    }
    in->root = Parser(doc).parse();
    read_all(in);
    in->ok = true;
  } catch (const std::exception &e) {
    in->err = e.what();
    if (!out) delete in;
    return CIL_ERR_CONFIG;
  }
  if (!out) delete in;
  return CIL_OK;
}

cil_status cil_input_config(const cil_input *in, cil_config *cfg, cil_colony_params *params, cil_run_info *run) {
  if (!in || !in->ok) return CIL_ERR_STATE;
  if (in->nelem != 2) {
    const_cast<cil_input *>(in)->err = "the run describes single-element cells: use cil_input_cycle_config";
    return CIL_ERR_STATE;
  }
  if (cfg) *cfg = in->cfg;
  if (params) *params = in->p;
  if (run) *run = in->run;
  return CIL_OK;
}

cil_status cil_input_initial_state(const cil_input *in, cil_colony_view *v) {
  if (!in || !in->ok || in->nelem != 2) return CIL_ERR_STATE;
  cil_input *m = const_cast<cil_input *>(in);
  if (!v || !v->pos || !v->sigma || !v->t0 || !v->tswitch) {
    m->err = "cil_input_initial_state: NULL arrays";
    return CIL_ERR_CONFIG;
  }
  const int n = in->ncells, D = in->dim;
  v->ncells = n;
  v->ts = 0;
  if (v->capacity < n) {
    m->err = "cil_input_initial_state: the view holds fewer cells than the initial configuration";
    return CIL_ERR_CAPACITY;
  }
  cil::HostRng rng;
  rng.seed(static_cast<uint32_t>(in->run.seed));  // Random::init(seed), readRunTime
  if (in->init_kind == "RANDOM") random_positions(rng, in, v->pos);
  else std::memcpy(v->pos, in->json_pos.data(), sizeof(double) * in->json_pos.size());
  // initializeCellStatus (CIL.cuh:253-330)
  for (int i = 0; i < n; ++i) {
    v->t0[i] = 0;
    v->tswitch[i] = -1;
    v->sigma[2 * i] = in->sigma[0];
    v->sigma[2 * i + 1] = in->sigma[1];
  }
  // cell states: what INIT read, else undefined (Colony.cpp:248); a dividing species turns an
  // undefined cell crawling or dividing with its time span (CIL.cuh:279-290)
  if (v->cell_state)
    for (int i = 0; i < n; ++i)
      v->cell_state[i] = static_cast<size_t>(i) < in->h5_state.size() ? in->h5_state[i] : 2;
  if (in->divide) {
    const double p_mig = in->tau_mig[0] / (in->tau_mig[0] + in->tau_div[0]);
    for (int i = 0; i < n; ++i) {
      int span;
      bool crawl = true;
      if (in->const_force) span = time_span(rng, in->tau_mig, in->dt);
      else if (rng.uniform0x(1.0) <= p_mig) span = time_span(rng, in->tau_mig, in->dt);
      else {
        span = time_span(rng, in->tau_div, in->dt);
        crawl = false;
      }
      if (v->cell_state && v->cell_state[i] == 2) v->cell_state[i] = crawl ? 1 : 0;
      (void)rng.uniform0x(1);  // theta, the cycle phase of the single-element model
      span -= nint(rng.uniform0x(static_cast<double>(span))) - 1;
      v->tswitch[i] = v->t0[i] + span;
    }
  }
  if (in->init_kind == "RANDOM") random_positions(rng, in, v->pos);  // the second readInit
  if (in->h5_all)  // the second readInit of H5 ALL: the file's diameters (velocities, phases and
                   // activities have no place in the two-element step)
    for (int i = 0; i < 2 * n; ++i) v->sigma[i] = in->h5_sigma[i];
  // initializeColony: positions must lie in the box along periodic axes (CIL.cuh:52-66)
  for (int i = 0; i < 2 * n; ++i)
    for (int d = 0; d < D; ++d) {
      const double r = v->pos[static_cast<size_t>(i) * D + d];
      if (std::isnan(r) || (in->pbc[d] && !(r >= 0.0 && r < in->box[d]))) {
        m->err = "Input Positions Out of Bounds! (cell " + std::to_string(i / 2) + ", element " +
                 std::to_string(i % 2) + ", axis " + std::to_string(d) + ")";
        return CIL_ERR_CONFIG;
      }
    }
  return CIL_OK;
}

int32_t cil_input_elements(const cil_input *in) { return in && in->ok ? in->nelem : 0; }

cil_status cil_input_cycle_config(const cil_input *in, cil_cycle_params *params, cil_run_info *run) {
  if (!in || !in->ok) return CIL_ERR_STATE;
  if (in->nelem != 1) {
    const_cast<cil_input *>(in)->err = "the run describes two-element cells: use cil_input_config";
    return CIL_ERR_STATE;
  }
  if (params) *params = in->cyc;
  if (run) *run = in->run;
  return CIL_OK;
}

cil_status cil_input_cycle_initial_state(const cil_input *in, cil_cycle_view *v) {
  if (!in || !in->ok) return CIL_ERR_STATE;
  cil_input *m = const_cast<cil_input *>(in);
  if (in->nelem != 1) {
    m->err = "the run describes two-element cells: use cil_input_initial_state";
    return CIL_ERR_STATE;
  }
  if (!v || !v->pos || !v->sigma || !v->sigma_t || !v->theta || !v->rho || !v->angvel) {
    m->err = "cil_input_cycle_initial_state: NULL arrays";
    return CIL_ERR_CONFIG;
  }
  const int n = in->ncells, D = in->dim;
  v->ncells = n;
  v->ts = 0;
  if (v->capacity < n) {
    m->err = "cil_input_cycle_initial_state: the view holds fewer cells than the initial configuration";
    return CIL_ERR_CAPACITY;
  }
  const cil_cycle_params &q = in->cyc;
  cil::HostRng rng;
  rng.seed(static_cast<uint32_t>(in->run.seed));
  auto positions = [&]() {  // Input.cpp:736-757 with one element: a uniform position per cell
    for (int i = 0; i < n; ++i)
      for (int d = 0; d < D; ++d) v->pos[static_cast<size_t>(i) * D + d] = rng.uniform0x(in->box[d]);
  };
  if (in->init_kind == "RANDOM") positions();
  else std::memcpy(v->pos, in->json_pos.data(), sizeof(double) * in->json_pos.size());
  // initializeCellStatus (CIL.cuh:253-330): every cell dividing, its cycle speed from the span
  const double tau[2] = {q.tau_div_mu, q.tau_div_sigma};
  for (int i = 0; i < n; ++i) {
    v->sigma[i] = q.sigma_core;
    v->sigma_t[i] = q.sigma_core;
    v->rho[i] = 1.0;
    v->theta[i] = -1.0;
    v->angvel[i] = -1.0;
    if (q.divide) {
      (void)rng.uniform0x(1.0);  // the migration test, probability 0 here
      int span = time_span(rng, tau, in->dt);
      v->angvel[i] = 1.0 / span;
      v->theta[i] = rng.uniform0x(1);
      span -= nint(rng.uniform0x(static_cast<double>(span))) - 1;
    }
  }
  if (in->init_kind == "RANDOM") positions();  // the second readInit
  if (in->h5_all) {  // the second readInit of H5 ALL replaces the drawn status (Input.cpp:711-719)
    for (int i = 0; i < n; ++i) {
      if (q.divide && in->h5_state[i] != 0) {
        m->err = "INIT H5: cell " + std::to_string(i) + " is not in the dividing state (crawling cells never "
                 "re-enter the single-element cycle)";
        return CIL_ERR_CONFIG;
      }
      v->sigma[i] = in->h5_sigma[i];
      v->sigma_t[i] = in->h5_sigma[i];
      v->theta[i] = in->h5_theta[i];
      v->rho[i] = in->h5_rho[i];
      if (v->vel)
        for (int d = 0; d < D; ++d)
          v->vel[static_cast<size_t>(i) * D + d] = in->h5_vel[static_cast<size_t>(i) * D + d];
    }
  }
  for (int i = 0; i < n; ++i)
    for (int d = 0; d < D; ++d) {
      const double r = v->pos[static_cast<size_t>(i) * D + d];
      if (std::isnan(r) || (in->pbc[d] && !(r >= 0.0 && r < in->box[d]))) {
        m->err = "Input Positions Out of Bounds! (cell " + std::to_string(i) + ", axis " + std::to_string(d) + ")";
        return CIL_ERR_CONFIG;
      }
    }
  return CIL_OK;
}

void cil_input_last_error(const cil_input *in, char *buf, size_t len) {
  if (!buf || len == 0) return;
  snprintf(buf, len, "%s", in ? in->err.c_str() : "");
}

void cil_input_free(cil_input *in) { delete in; }

}  // extern "C"
