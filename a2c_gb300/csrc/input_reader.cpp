// Reader of the reference's input-file syntax (the grammar of
// parser/Parser.y and the tokens of parser/Lexer.l), hand-written: the
// reference generates its parser with bison/flex.
//
//   File      : { Assignment | Group } ( end-of-file | "end" )
//   Assignment: Assignable '=' ( Symbol | IntExpr | DblExpr | String ) ';'
//   Group     : "under" Assignable '{' { Assignment | Group } '}'
//   Assignable: Symbol { '.' Symbol | '[' IntExpr ']' }
//   IntExpr / DblExpr: constants, ( ), + - * / with * / binding tighter;
//                      int op int is an int (C division), anything with a
//                      double is a double
// Tokens as Lexer.l: // and /* */ comments; a sign directly before digits
// belongs to the number ("2 -5" is two constants, a syntax error as in the
// reference); d/D exponents; strings of [A-z0-9._/-] in double quotes.
//
// Every assignment is stored under its full path (the under-blocks'
// paths, then the assignable), e.g. "Material[0].InteratomicPotential.
// CutOffDistance".  The fields the evaluator and the DMD loop use are then
// read into a2c_input with the reference's defaults (IoData.cpp); the rest
// of a full input file (geometry, species, ...) is parsed and counted.
#include <algorithm>
#include <cctype>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "a2c_gpp.h"

namespace {

enum Tok { T_EOF, T_END, T_UNDER, T_SYM, T_INT, T_DBL, T_STR, T_CHAR };

struct Token {
  Tok t;
  std::string s;  // symbol / string text
  long long i = 0;
  double d = 0.0;
  char c = 0;
  int line = 1;
};

struct Value {
  enum Kind { INT, DBL, STR, SYM } kind = INT;
  long long i = 0;
  double d = 0.0;
  std::string s;
};

struct Error {
  std::string msg;
};

class Lexer {
 public:
  explicit Lexer(const std::string &src) : s_(src) {}
  Token next() {
    for (;;) {
      if (p_ >= s_.size()) return tok(T_EOF);
      const char c = s_[p_];
      if (c == '\n') {
        ++line_;
        ++p_;
      } else if (c == ' ' || c == '\t' || c == '\r') {
        ++p_;
      } else if (c == '/' && p_ + 1 < s_.size() && s_[p_ + 1] == '/') {
        while (p_ < s_.size() && s_[p_] != '\n') ++p_;
      } else if (c == '/' && p_ + 1 < s_.size() && s_[p_ + 1] == '*') {
        p_ += 2;
        while (p_ + 1 < s_.size() && !(s_[p_] == '*' && s_[p_ + 1] == '/')) {
          if (s_[p_] == '\n') ++line_;
          ++p_;
        }
        if (p_ + 1 >= s_.size()) throw Error{"unterminated comment near line " + std::to_string(line_)};
        p_ += 2;
      } else {
        break;
      }
    }
    const char c = s_[p_];
    if (c == '"') {
      size_t q = p_ + 1;
      while (q < s_.size() && strchar(s_[q])) ++q;
      if (q >= s_.size() || s_[q] != '"') throw Error{"bad string near line " + std::to_string(line_)};
      Token t = tok(T_STR);
      t.s = s_.substr(p_ + 1, q - p_ - 1);
      p_ = q + 1;
      return t;
    }
    if (std::isdigit((unsigned char)c) || c == '.' ||
        ((c == '+' || c == '-') && p_ + 1 < s_.size() &&
         (std::isdigit((unsigned char)s_[p_ + 1]) ||
          (s_[p_ + 1] == '.' && p_ + 2 < s_.size() && std::isdigit((unsigned char)s_[p_ + 2]))))) {
      Token t;
      if (number(t)) return t;
    }
    if (std::isalpha((unsigned char)c) || c == '_') {
      size_t q = p_;
      while (q < s_.size() && (std::isalnum((unsigned char)s_[q]) || s_[q] == '_')) ++q;
      const std::string w = s_.substr(p_, q - p_);
      p_ = q;
      if (w == "end") return tok(T_END);
      if (w == "under") return tok(T_UNDER);
      Token t = tok(T_SYM);
      t.s = w;
      return t;
    }
    if (std::strchr("-+*[]^{}=,():;./", c)) {
      Token t = tok(T_CHAR);
      t.c = c;
      ++p_;
      return t;
    }
    throw Error{std::string("unexpected character '") + c + "' near line " + std::to_string(line_)};
  }
  int line() const { return line_; }

 private:
  static bool strchar(char ch) {
    return (ch >= 'A' && ch <= 'z') || std::isdigit((unsigned char)ch) || ch == '.' || ch == '_' || ch == '/' ||
           ch == '-';
  }
  Token tok(Tok t) const {
    Token k;
    k.t = t;
    k.line = line_;
    return k;
  }
  // [+-]? digits [. digits*] [eEdD [+-]? digits] | [+-]? . digits [exp]
  bool number(Token &t) {
    size_t q = p_;
    if (s_[q] == '+' || s_[q] == '-') ++q;
    const size_t d0 = q;
    while (q < s_.size() && std::isdigit((unsigned char)s_[q])) ++q;
    bool dbl = false;
    const bool int_digits = q > d0;
    if (q < s_.size() && s_[q] == '.') {
      const size_t f0 = q + 1;
      size_t f = f0;
      while (f < s_.size() && std::isdigit((unsigned char)s_[f])) ++f;
      if (!int_digits && f == f0) return false;  // a lone '.'
      dbl = true;
      q = f;
    } else if (!int_digits) {
      return false;
    }
    if (q < s_.size() && std::strchr("eEdD", s_[q])) {
      size_t e = q + 1;
      if (e < s_.size() && (s_[e] == '+' || s_[e] == '-')) ++e;
      const size_t e0 = e;
      while (e < s_.size() && std::isdigit((unsigned char)s_[e])) ++e;
      if (e > e0) {
        dbl = true;
        q = e;
      }
    }
    std::string txt = s_.substr(p_, q - p_);
    for (char &ch : txt)
      if (ch == 'd' || ch == 'D') ch = 'e';
    t = tok(dbl ? T_DBL : T_INT);
    if (dbl) t.d = std::atof(txt.c_str());
    else t.i = std::atoll(txt.c_str());
    p_ = q;
    return true;
  }
  const std::string &s_;
  size_t p_ = 0;
  int line_ = 1;
};

class Parser {
 public:
  explicit Parser(const std::string &src) : lx_(src) { adv(); }
  std::map<std::string, Value> values;
  int assignments = 0;

  void file() {
    items();
    if (cur_.t != T_EOF && cur_.t != T_END) fail();
  }

 private:
  void adv() { cur_ = lx_.next(); }
  [[noreturn]] void fail() {
    throw Error{"syntax error near line " + std::to_string(cur_.line)};
  }
  bool is(char c) const { return cur_.t == T_CHAR && cur_.c == c; }
  void expect(char c) {
    if (!is(c)) fail();
    adv();
  }
  void items() {
    for (;;) {
      if (cur_.t == T_UNDER) {
        adv();
        std::string path = assignable();
        expect('{');
        under_.push_back(path);
        items();
        expect('}');
        under_.pop_back();
      } else if (cur_.t == T_SYM) {
        std::string path = assignable();
        expect('=');
        Value v;
        if (cur_.t == T_SYM) {
          v.kind = Value::SYM;
          v.s = cur_.s;
          adv();
        } else if (cur_.t == T_STR) {
          v.kind = Value::STR;
          v.s = cur_.s;
          adv();
        } else {
          v = expr();
        }
        expect(';');
        std::string key;
        for (const std::string &u : under_) key += u + ".";
        values[key + path] = v;
        ++assignments;
      } else {
        return;
      }
    }
  }
  std::string assignable() {
    if (cur_.t != T_SYM) fail();
    std::string p = cur_.s;
    adv();
    for (;;) {
      if (is('.')) {
        adv();
        if (cur_.t != T_SYM) fail();
        p += "." + cur_.s;
        adv();
      } else if (is('[')) {
        adv();
        Value i = expr();
        if (i.kind != Value::INT) fail();
        expect(']');
        p += "[" + std::to_string(i.i) + "]";
      } else {
        return p;
      }
    }
  }
  static Value arith(const Value &a, const Value &b, char op) {
    Value r;
    if (a.kind == Value::INT && b.kind == Value::INT) {
      r.kind = Value::INT;
      if (op == '/' && b.i == 0) throw Error{"integer division by zero"};
      r.i = op == '+' ? a.i + b.i : op == '-' ? a.i - b.i : op == '*' ? a.i * b.i : a.i / b.i;
    } else {
      r.kind = Value::DBL;
      const double x = a.kind == Value::INT ? (double)a.i : a.d, y = b.kind == Value::INT ? (double)b.i : b.d;
      r.d = op == '+' ? x + y : op == '-' ? x - y : op == '*' ? x * y : x / y;
    }
    return r;
  }
  Value expr() {  // left-associative + -
    Value v = term();
    while (is('+') || is('-')) {
      const char op = cur_.c;
      adv();
      v = arith(v, term(), op);
    }
    return v;
  }
  Value term() {  // left-associative * /
    Value v = atom();
    while (is('*') || is('/')) {
      const char op = cur_.c;
      adv();
      v = arith(v, atom(), op);
    }
    return v;
  }
  Value atom() {
    Value v;
    if (cur_.t == T_INT) {
      v.kind = Value::INT;
      v.i = cur_.i;
      adv();
    } else if (cur_.t == T_DBL) {
      v.kind = Value::DBL;
      v.d = cur_.d;
      adv();
    } else if (is('(')) {
      adv();
      v = expr();
      expect(')');
    } else {
      fail();
    }
    return v;
  }
  Lexer lx_;
  Token cur_;
  std::vector<std::string> under_;
};

bool get_num(const std::map<std::string, Value> &m, const char *key, double &out) {
  auto it = m.find(key);
  if (it == m.end()) return false;
  if (it->second.kind == Value::INT) out = (double)it->second.i;
  else if (it->second.kind == Value::DBL) out = it->second.d;
  else throw Error{std::string(key) + ": a number is expected"};
  return true;
}
bool get_int(const std::map<std::string, Value> &m, const char *key, int &out) {
  auto it = m.find(key);
  if (it == m.end()) return false;
  if (it->second.kind != Value::INT) throw Error{std::string(key) + ": an integer is expected"};
  out = (int)it->second.i;
  return true;
}
bool get_str(const std::map<std::string, Value> &m, const char *key, char *out, size_t n) {
  auto it = m.find(key);
  if (it == m.end()) return false;
  if (it->second.kind != Value::STR) throw Error{std::string(key) + ": a string is expected"};
  std::snprintf(out, n, "%s", it->second.s.c_str());
  return true;
}
// a token among names[k] -> codes[k]
bool get_tok(const std::map<std::string, Value> &m, const char *key, const std::vector<std::pair<const char *, int>> &opt,
             int &out) {
  auto it = m.find(key);
  if (it == m.end()) return false;
  if (it->second.kind != Value::SYM) throw Error{std::string(key) + ": a keyword is expected"};
  for (const auto &o : opt)
    if (it->second.s == o.first) {
      out = o.second;
      return true;
    }
  throw Error{std::string(key) + ": unknown keyword " + it->second.s};
}

void defaults(a2c_input *in) {
  std::memset(in, 0, sizeof(*in));
  in->T = 300.0;  // DiffusionData (IoData.cpp:628-635)
  in->nu = 0.0;
  in->Qm = 0.0;
  in->t_subsurf = 0.0;
  in->mubd = -2.0;
  in->eps = 1.0e-5;  // InteratomicPotentialData (IoData.cpp:514-519)
  in->rc = 5.35;
  in->dt = -1.0;  // TsData (IoData.cpp:683-689)
  in->max_time = 1e10;
  in->max_its = INT_MAX;
  in->cfl = 0.5;
  in->output_format = 1;  // OutputData (IoData.cpp:706-715): VTP, Medium, "solution"
  in->output_precision = 1;
  std::snprintf(in->output_solution, sizeof(in->output_solution), "solution");
  in->output_frequency = 0;
  in->output_interval = -1.0;
  for (int k = 0; k < 3; ++k) in->lattice_axes[4 * k] = 1.0;  // LatticeData (IoData.cpp:451-463)
}

}  // namespace

extern "C" a2c_status a2c_input_read(const char *path, a2c_input *in, char *errmsg, int errlen) {
  if (!path || !in) return A2C_ERR_INVALID;
  auto err = [&](const std::string &m) {
    if (errmsg && errlen > 0) std::snprintf(errmsg, (size_t)errlen, "%s", m.c_str());
    return A2C_ERR_INVALID;
  };
  std::ifstream f(path);
  if (!f) return err(std::string("cannot open ") + path);
  std::stringstream ss;
  ss << f.rdbuf();
  const std::string src = ss.str();
  defaults(in);
  try {
    Parser p(src);
    p.file();
    const auto &m = p.values;
    int used = 0;
    used += get_num(m, "Diffusion.Temperature", in->T);
    used += get_num(m, "Diffusion.AttemptFrequency", in->nu);
    used += get_num(m, "Diffusion.ActivationEnergy", in->Qm);
    used += get_num(m, "Diffusion.SubsurfaceThickness", in->t_subsurf);
    used += get_num(m, "Diffusion.SoluteChemicalPotential", in->mubd);
    used += get_num(m, "Material[0].InteratomicPotential.Tolerance", in->eps);
    used += get_num(m, "Material[0].InteratomicPotential.CutOffDistance", in->rc);
    used += get_str(m, "Material[0].InteratomicPotential.File", in->potential_file, sizeof(in->potential_file));
    used += get_num(m, "Time.TimeStep", in->dt);
    used += get_num(m, "Time.MaxTime", in->max_time);
    used += get_int(m, "Time.MaxIts", in->max_its);
    used += get_num(m, "Time.CFL", in->cfl);
    int fmt = 0;
    if (get_tok(m, "Output.Format", {{"VTP", 1}, {"XYZ", 2}, {"VTP_and_XYZ", 3}, {"XYZ_and_VTP", 3}}, fmt)) {
      in->output_format = fmt;
      ++used;
    }
    used += get_tok(m, "Output.Precision", {{"Low", 0}, {"Medium", 1}, {"High", 2}}, in->output_precision);
    used += get_str(m, "Output.Prefix", in->output_prefix, sizeof(in->output_prefix));
    used += get_str(m, "Output.Solution", in->output_solution, sizeof(in->output_solution));
    used += get_int(m, "Output.Frequency", in->output_frequency);
    used += get_num(m, "Output.TimeInterval", in->output_interval);
    const char *ax[9] = {"OAx", "OAy", "OAz", "OBx", "OBy", "OBz", "OCx", "OCy", "OCz"};
    for (int k = 0; k < 9; ++k) used += get_num(m, (std::string("Lattice[0].") + ax[k]).c_str(), in->lattice_axes[k]);
    const char *org[3] = {"Ox", "Oy", "Oz"};
    for (int k = 0; k < 3; ++k) used += get_num(m, (std::string("Lattice[0].") + org[k]).c_str(), in->lattice_origin[k]);
    const char *per[3] = {"PeriodicOA", "PeriodicOB", "PeriodicOC"};
    for (int k = 0; k < 3; ++k)
      used += get_tok(m, (std::string("Lattice[0].") + per[k]).c_str(), {{"False", 0}, {"True", 1}},
                      in->lattice_periodic[k]);
    in->n_assignments = p.assignments;
    in->n_used = used;
  } catch (const Error &e) {
    return err(e.msg);
  }
  if (errmsg && errlen > 0) errmsg[0] = 0;
  return A2C_OK;
}

namespace {

// Indices k of the blocks "<prefix><name>[k]." present in the file.
std::vector<int> block_ids(const std::map<std::string, Value> &m, const std::string &prefix, const char *name) {
  const std::string head = prefix + name + "[";
  std::vector<int> ids;
  for (auto it = m.lower_bound(head); it != m.end() && it->first.compare(0, head.size(), head) == 0; ++it) {
    const size_t close = it->first.find(']', head.size());
    if (close == std::string::npos || close == head.size()) continue;
    const std::string num = it->first.substr(head.size(), close - head.size());
    if (num.find_first_not_of("0123456789") != std::string::npos) continue;
    const int k = std::atoi(num.c_str());
    if (ids.empty() || ids.back() != k) ids.push_back(k);
  }
  std::sort(ids.begin(), ids.end());
  ids.erase(std::unique(ids.begin(), ids.end()), ids.end());
  return ids;
}

const std::vector<std::pair<const char *, int>> kInclusion = {{"Override", 0}, {"Intersection", 1}, {"Union", 2}};
const std::vector<std::pair<const char *, int>> kSide = {{"Interior", 0}, {"Exterior", 1}};
const std::vector<std::pair<const char *, int>> kOnOff = {{"Off", 0}, {"On", 1}};

// The geometry blocks under `prefix` (Plane, CylinderAndCone,
// CylinderWithSphericalCaps, Sphere, Parallelepiped, Spheroid; IoData.cpp:
// 9-330, names and defaults) into geoms[ng ..]; returns the new count.
int read_geometries(const std::map<std::string, Value> &m, const std::string &prefix, a2c_geometry *geoms,
                    int max_geoms, int ng) {
  auto key = [&](const std::string &rest) { return prefix + rest; };
  auto next = [&](int type) -> a2c_geometry & {
    if (ng >= max_geoms) throw Error{"more geometries than the array holds"};
    a2c_geometry &g = geoms[ng++];
    std::memset(&g, 0, sizeof(g));
    g.type = type;
    return g;
  };
  auto common = [&](a2c_geometry &g, const std::string &G, bool sided) {
    get_int(m, key(G + "OperationOrder").c_str(), g.order);
    get_tok(m, key(G + "Inclusion").c_str(), kInclusion, g.inclusion);
    if (sided) get_tok(m, key(G + "Side").c_str(), kSide, g.exterior);
  };
  auto nums = [&](a2c_geometry &g, const std::string &G, std::initializer_list<const char *> names, int at) {
    for (const char *nm : names) get_num(m, key(G + nm).c_str(), g.p[at++]);
  };
  char spec[256] = {0};
  get_str(m, key("CustomGeometry.GeometrySpecifier").c_str(), spec, sizeof(spec));
  if (spec[0])  // a plug-in loaded with dlopen (SpaceInitializer.cpp:150-178)
    throw Error{prefix + "CustomGeometry: geometry plug-ins are not supported"};
  for (int k : block_ids(m, prefix, "Plane")) {
    const std::string G = "Plane[" + std::to_string(k) + "].";
    a2c_geometry &g = next(A2C_GEOM_PLANE);
    nums(g, G, {"Point_x", "Point_y", "Point_z", "Normal_x", "Normal_y", "Normal_z"}, 0);
    common(g, G, false);
  }
  for (int k : block_ids(m, prefix, "CylinderAndCone")) {
    const std::string G = "CylinderAndCone[" + std::to_string(k) + "].";
    a2c_geometry &g = next(A2C_GEOM_CYLINDER_CONE);
    g.p[5] = 1.0;   // axis (0, 0, 1)
    g.p[6] = 1.0;   // radius
    g.p[8] = 45.0;  // opening angle
    nums(g, G, {"BaseCenter_x", "BaseCenter_y", "BaseCenter_z", "Axis_x", "Axis_y", "Axis_z", "CylinderRadius",
                "CylinderHeight", "ConeOpeningAngleInDegrees", "ConeHeight"},
         0);
    common(g, G, true);
  }
  for (int k : block_ids(m, prefix, "CylinderWithSphericalCaps")) {
    const std::string G = "CylinderWithSphericalCaps[" + std::to_string(k) + "].";
    a2c_geometry &g = next(A2C_GEOM_CYLINDER_SPHERE);
    g.p[5] = 1.0;
    g.p[6] = 1.0;
    nums(g, G, {"BaseCenter_x", "BaseCenter_y", "BaseCenter_z", "Axis_x", "Axis_y", "Axis_z", "CylinderRadius",
                "CylinderHeight"},
         0);
    int front = 0, back = 0;
    get_tok(m, key(G + "FrontSphericalCap").c_str(), kOnOff, front);
    get_tok(m, key(G + "BackSphericalCap").c_str(), kOnOff, back);
    g.p[8] = front;
    g.p[9] = back;
    common(g, G, true);
  }
  for (int k : block_ids(m, prefix, "Sphere")) {
    const std::string G = "Sphere[" + std::to_string(k) + "].";
    a2c_geometry &g = next(A2C_GEOM_SPHERE);
    g.p[3] = -1.0;
    nums(g, G, {"Center_x", "Center_y", "Center_z", "Radius"}, 0);
    common(g, G, true);
  }
  for (int k : block_ids(m, prefix, "Parallelepiped")) {
    const std::string G = "Parallelepiped[" + std::to_string(k) + "].";
    a2c_geometry &g = next(A2C_GEOM_PARALLELEPIPED);
    nums(g, G, {"Px", "Py", "Pz", "Ax", "Ay", "Az", "Bx", "By", "Bz", "Cx", "Cy", "Cz"}, 0);
    common(g, G, true);
  }
  for (int k : block_ids(m, prefix, "Spheroid")) {
    const std::string G = "Spheroid[" + std::to_string(k) + "].";
    a2c_geometry &g = next(A2C_GEOM_SPHEROID);
    nums(g, G, {"Center_x", "Center_y", "Center_z", "Axis_x", "Axis_y", "Axis_z", "SemiLength", "Radius"}, 0);
    common(g, G, true);
  }
  return ng;
}

}  // namespace

// Lattice[id] of an input file (LatticeData, LatticeSiteData and the
// geometry data of IoData.cpp:9-470: names and defaults).
extern "C" a2c_status a2c_input_lattice(const char *path, int lattice_id, a2c_lattice_desc *desc,
                                        a2c_site_group *sites, int max_sites, a2c_geometry *geoms, int max_geoms,
                                        char *errmsg, int errlen) {
  if (!path || !desc || lattice_id < 0 || max_sites < 0 || max_geoms < 0 || (max_sites > 0 && !sites) ||
      (max_geoms > 0 && !geoms))
    return A2C_ERR_INVALID;
  auto err = [&](const std::string &msg) {
    if (errmsg && errlen > 0) std::snprintf(errmsg, (size_t)errlen, "%s", msg.c_str());
    return A2C_ERR_INVALID;
  };
  std::ifstream f(path);
  if (!f) return err(std::string("cannot open ") + path);
  std::stringstream ss;
  ss << f.rdbuf();
  const std::string src = ss.str();  // the lexer reads it in place
  try {
    Parser p(src);
    p.file();
    const auto &m = p.values;
    const std::string L = "Lattice[" + std::to_string(lattice_id) + "].";
    auto key = [&](const std::string &rest) { return L + rest; };
    std::memset(desc, 0, sizeof(*desc));
    const char *ax[9] = {"OAx", "OAy", "OAz", "OBx", "OBy", "OBz", "OCx", "OCy", "OCz"};
    for (int k = 0; k < 9; ++k) {
      desc->abc[k] = (k % 4 == 0) ? 1.0 : 0.0;
      get_num(m, key(ax[k]).c_str(), desc->abc[k]);
    }
    const char *org[3] = {"Ox", "Oy", "Oz"};
    for (int k = 0; k < 3; ++k) get_num(m, key(org[k]).c_str(), desc->origin[k]);
    const char *per[3] = {"PeriodicOA", "PeriodicOB", "PeriodicOC"};
    for (int k = 0; k < 3; ++k) get_tok(m, key(per[k]).c_str(), {{"False", 0}, {"True", 1}}, desc->periodic[k]);
    get_num(m, key("MinDistance").c_str(), desc->dmin);
    // sites: ids 0 .. n-1 (LatticeStructure.cpp:80-87)
    const std::vector<int> sid = block_ids(m, L, "Site");
    if ((int)sid.size() > max_sites) throw Error{"more sites than the arrays hold"};
    for (int s = 0; s < (int)sid.size(); ++s) {
      if (sid[s] != s) throw Error{"site ids must be 0 .. n-1"};
      const std::string S = "Site[" + std::to_string(s) + "].";
      a2c_site_group &g = sites[s];
      g.l[0] = g.l[1] = g.l[2] = -1.0;
      g.materialid = -1;
      g.tag = 0;
      g.atomic_frequency = -1.0;
      g.mean_displacement[0] = g.mean_displacement[1] = g.mean_displacement[2] = 0.0;
      g.x = -1.0e-3;
      get_num(m, key(S + "La").c_str(), g.l[0]);
      get_num(m, key(S + "Lb").c_str(), g.l[1]);
      get_num(m, key(S + "Lc").c_str(), g.l[2]);
      get_int(m, key(S + "MaterialID").c_str(), g.materialid);
      get_int(m, key(S + "Tag").c_str(), g.tag);
      get_num(m, key(S + "AtomicFrequency").c_str(), g.atomic_frequency);
      get_num(m, key(S + "MeanDisplacementX").c_str(), g.mean_displacement[0]);
      get_num(m, key(S + "MeanDisplacementY").c_str(), g.mean_displacement[1]);
      get_num(m, key(S + "MeanDisplacementZ").c_str(), g.mean_displacement[2]);
      get_num(m, key(S + "LocalSpecies[0].MolarFraction").c_str(), g.x);
    }
    desc->nsites = (int)sid.size();
    desc->sites = sites;
    // geometries, each with its defaults
    const int ng = read_geometries(m, L, geoms, max_geoms, 0);
    desc->ngeom = ng;
    desc->geoms = geoms;
  } catch (const Error &e) {
    return err(e.msg);
  }
  if (errmsg && errlen > 0) errmsg[0] = 0;
  return A2C_OK;
}

// Material[m].MaterialName (MaterialData, IoData.cpp:538-560).
extern "C" a2c_status a2c_input_material_names(const char *path, char *names, int max_materials, int name_len,
                                               int *n_materials, char *errmsg, int errlen) {
  if (!path || !n_materials || max_materials < 0 || name_len < 1 || (max_materials > 0 && !names))
    return A2C_ERR_INVALID;
  auto err = [&](const std::string &msg) {
    if (errmsg && errlen > 0) std::snprintf(errmsg, (size_t)errlen, "%s", msg.c_str());
    return A2C_ERR_INVALID;
  };
  std::ifstream f(path);
  if (!f) return err(std::string("cannot open ") + path);
  std::stringstream ss;
  ss << f.rdbuf();
  const std::string src = ss.str();  // the lexer reads it in place
  try {
    Parser p(src);
    p.file();
    const auto &m = p.values;
    const std::vector<int> ids = block_ids(m, "", "Material");
    int n = 0;
    for (int k : ids) n = std::max(n, k + 1);
    if (n > max_materials) throw Error{"more materials than the array holds"};
    for (int k = 0; k < n; ++k) {
      char *out = names + (size_t)k * (size_t)name_len;
      out[0] = 0;
      get_str(m, ("Material[" + std::to_string(k) + "].MaterialName").c_str(), out, (size_t)name_len);
    }
    *n_materials = n;
  } catch (const Error &e) {
    return err(e.msg);
  }
  if (errmsg && errlen > 0) errmsg[0] = 0;
  return A2C_OK;
}

// RegionalInitialCondition[k] blocks (RegionalIcData, IoData.cpp:578-624).
extern "C" a2c_status a2c_input_regions(const char *path, a2c_region *regions, int max_regions,
                                        a2c_geometry *geoms, int max_geoms, int *n_regions, char *errmsg,
                                        int errlen) {
  if (!path || !n_regions || max_regions < 0 || max_geoms < 0 || (max_regions > 0 && !regions) ||
      (max_geoms > 0 && !geoms))
    return A2C_ERR_INVALID;
  auto err = [&](const std::string &msg) {
    if (errmsg && errlen > 0) std::snprintf(errmsg, (size_t)errlen, "%s", msg.c_str());
    return A2C_ERR_INVALID;
  };
  std::ifstream f(path);
  if (!f) return err(std::string("cannot open ") + path);
  std::stringstream ss;
  ss << f.rdbuf();
  const std::string src = ss.str();  // the lexer reads it in place
  try {
    Parser p(src);
    p.file();
    const auto &m = p.values;
    const std::vector<int> ids = block_ids(m, "", "RegionalInitialCondition");
    if ((int)ids.size() > max_regions) throw Error{"more regions than the array holds"};
    int ng = 0;
    for (int k = 0; k < (int)ids.size(); ++k) {
      if (ids[k] != k) throw Error{"RegionalInitialCondition ids must be 0 .. n-1"};
      const std::string R = "RegionalInitialCondition[" + std::to_string(k) + "].";
      a2c_region &r = regions[k];
      std::memset(&r, 0, sizeof(r));
      r.lattice_id = r.materialid = r.siteid = -1;
      r.atomic_frequency = -1.0;
      r.x = -1.0e-3;
      get_int(m, (R + "LatticeID").c_str(), r.lattice_id);
      get_int(m, (R + "MaterialID").c_str(), r.materialid);
      get_int(m, (R + "SiteID").c_str(), r.siteid);
      get_int(m, (R + "Tag").c_str(), r.tag);
      get_num(m, (R + "AtomicFrequency").c_str(), r.atomic_frequency);
      get_num(m, (R + "MeanDisplacementX").c_str(), r.mean_displacement[0]);
      get_num(m, (R + "MeanDisplacementY").c_str(), r.mean_displacement[1]);
      get_num(m, (R + "MeanDisplacementZ").c_str(), r.mean_displacement[2]);
      get_num(m, (R + "LocalSpecies[0].MolarFraction").c_str(), r.x);
      const int ng1 = read_geometries(m, R, geoms, max_geoms, ng);
      r.ngeom = ng1 - ng;
      r.geoms = geoms + ng;
      ng = ng1;
    }
    *n_regions = (int)ids.size();
  } catch (const Error &e) {
    return err(e.msg);
  }
  if (errmsg && errlen > 0) errmsg[0] = 0;
  return A2C_OK;
}

// The evaluator parameters an input file sets: temperature, FD step and
// cutoff (the lattice spacing, box and precision are the caller's).
extern "C" a2c_status a2c_input_apply(const a2c_input *in, a2c_gpp_params *p) {
  if (!in || !p) return A2C_ERR_INVALID;
  p->T = in->T;
  p->eps = in->eps;
  p->rc = in->rc;
  return A2C_OK;
}
