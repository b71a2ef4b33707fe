// deck.cpp -- control-file reader: the subset of BookLeaf's namelists the
// hot path needs, with the reference's defaults and rationalisation.
//
//   CONTROL              setup_read.f90:113-253 (defaults time_config.f90,
//                        hydro_config.f90:32-82; rationalise
//                        hydro_config.f90:292-414)
//   ALE                  setup_read.f90:255-431, ale_config.f90:31-117, 511-551
//   CUTOFF               setup_read.f90:467-507, global_config.f90:32-42,
//                        eos_config.f90:31-60
//   EOS                  setup_read.f90:509-589, eos_config.f90:163-226
//
// Accepted syntax is what the reference's decks use: `name = v`,
// `name(i) = v`, `name(i,j) = v`, array sections with `:` or `a:b` filled
// in column-major order by a value list, quoted strings, logicals
// .TRUE./.FALSE., `!` comments.  Unknown groups are ignored.
#include <algorithm>
#include <cctype>
#include <cfloat>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <regex>
#include <sstream>

#include "blh.hpp"

namespace blh {

namespace {

constexpr int LN = 100;  // setup_read.f90:31, setup_IC.f90:82
constexpr int LI = 100;  // setup_mesh.F90:115

std::string upper(std::string s) {
  for (auto& c : s) c = (char)std::toupper((unsigned char)c);
  return s;
}
std::string lower(std::string s) {
  for (auto& c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}
std::string strip(const std::string& s) {
  size_t a = 0, b = s.size();
  while (a < b && std::isspace((unsigned char)s[a])) a++;
  while (b > a && std::isspace((unsigned char)s[b - 1])) b--;
  return s.substr(a, b - a);
}

std::string strip_comments(const std::string& text) {
  std::string out;
  std::istringstream in(text);
  std::string line;
  bool first = true;
  while (std::getline(in, line)) {
    char q = 0;
    size_t cut = line.size();
    for (size_t i = 0; i < line.size(); i++) {
      const char ch = line[i];
      if (q) {
        if (ch == q) q = 0;
      } else if (ch == '\'' || ch == '"') {
        q = ch;
      } else if (ch == '!') {
        cut = i;
        break;
      }
    }
    if (!first) out += '\n';
    out += line.substr(0, cut);
    first = false;
  }
  return out;
}

struct Item {
  char kind;  // 'S' string, 'W' word, '=' equals
  std::string s;
};

Value parse_value(const Item& it) {
  if (it.kind == 'S') return Value::str(it.s);
  const std::string& s = it.s;
  const std::string u = upper(s);
  if (u == ".TRUE." || u == "T" || u == ".T." || u == "TRUE") return Value::boolean(true);
  if (u == ".FALSE." || u == "F" || u == ".F." || u == "FALSE") return Value::boolean(false);
  static const std::regex int_re("[+-]?[0-9]+");
  if (std::regex_match(s, int_re)) return Value::integer(std::strtoll(s.c_str(), nullptr, 10));
  std::string t = s;
  for (auto& c : t)
    if (c == 'd' || c == 'D') c = 'e';
  static const std::regex real_re(
      "[+-]?(([0-9]+\\.?[0-9]*)|(\\.[0-9]+))([eE][+-]?[0-9]+)?|[+-]?(inf|infinity|nan)",
      std::regex::icase);
  if (std::regex_match(t, real_re)) return Value::real(std::strtod(t.c_str(), nullptr));
  return Value::str(s);
}

// key = values pairs of a group body
std::vector<std::pair<std::string, std::vector<Item>>> tokens(const std::string& body) {
  std::vector<Item> items;
  std::string cur;
  size_t i = 0, n = body.size();
  auto flush = [&]() {
    const std::string t = strip(cur);
    if (!t.empty()) items.push_back({'W', t});
    cur.clear();
  };
  while (i < n) {
    const char ch = body[i];
    if (ch == '\'' || ch == '"') {
      const size_t j = body.find(ch, i + 1);
      if (j == std::string::npos) throw DeckError("ERROR: unterminated string in namelist");
      items.push_back({'S', body.substr(i + 1, j - i - 1)});
      i = j + 1;
      continue;
    }
    if (ch == '(') {
      const size_t j = body.find(')', i);
      if (j == std::string::npos) throw DeckError("ERROR: unbalanced parenthesis in namelist");
      cur += body.substr(i, j - i + 1);
      i = j + 1;
      continue;
    }
    if (ch == ',' || ch == '\n' || ch == '\t' || ch == ' ' || ch == '\r') {
      flush();
      i++;
      continue;
    }
    if (ch == '=') {
      flush();
      items.push_back({'=', "="});
      i++;
      continue;
    }
    cur += ch;
    i++;
  }
  flush();
  std::vector<std::pair<std::string, std::vector<Item>>> out;
  size_t k = 0;
  while (k < items.size()) {
    if (k + 1 < items.size() && items[k + 1].kind == '=') {
      const std::string key = items[k].s;
      k += 2;
      std::vector<Item> vals;
      while (k < items.size() && !(k + 1 < items.size() && items[k + 1].kind == '=')) {
        vals.push_back(items[k]);
        k++;
      }
      out.emplace_back(key, vals);
    } else {
      throw DeckError("ERROR: namelist syntax near '" + items[k].s + "'");
    }
  }
  return out;
}

// index tuples (1-based) of an array section, column-major order
std::vector<std::vector<int>> indices(const std::string& sub, const std::vector<int>& ext) {
  std::vector<std::string> parts;
  {
    std::string p;
    for (char c : sub) {
      if (c == ',') {
        parts.push_back(strip(p));
        p.clear();
      } else {
        p += c;
      }
    }
    parts.push_back(strip(p));
  }
  std::vector<std::vector<int>> ranges;
  for (size_t d = 0; d < parts.size(); d++) {
    const int e = d < ext.size() ? ext[d] : LN;
    const std::string& p = parts[d];
    std::vector<int> r;
    if (p == ":") {
      for (int v = 1; v <= e; v++) r.push_back(v);
    } else if (p.find(':') != std::string::npos) {
      const size_t c = p.find(':');
      const std::string a = strip(p.substr(0, c)), b = strip(p.substr(c + 1));
      const int lo = a.empty() ? 1 : std::atoi(a.c_str());
      const int hi = b.empty() ? e : std::atoi(b.c_str());
      for (int v = lo; v <= hi; v++) r.push_back(v);
    } else {
      r.push_back(std::atoi(p.c_str()));
    }
    ranges.push_back(r);
  }
  std::vector<std::vector<int>> idx(1);
  for (const auto& r : ranges) {  // the first dimension varies fastest
    std::vector<std::vector<int>> next;
    for (int v : r)
      for (const auto& prev : idx) {
        auto t = prev;
        t.push_back(v);
        next.push_back(t);
      }
    idx.swap(next);
  }
  return idx;
}

std::vector<int> extents(const std::string& var, size_t ndim) {
  if (var == "region_side") return {LI, 4, LI};
  if (var == "region_dim") return {LI, 2};
  if (var == "segment_pos") return {LI, 8};
  if (var == "eos_param") return {6, LN};
  if (var == "kinematic_param") return {3, LN};
  if (var == "shape_param") return {LN, 5};
  if (var == "patch_trigger") return {LN, LN};
  return std::vector<int>(ndim, LN);
}

}  // namespace

// ------------------------------------------------------------------ values

double Value::as_real() const {
  switch (kind) {
    case REAL: return d;
    case INT: return (double)i;
    case BOOL: return b ? 1.0 : 0.0;
    default: throw DeckError("ERROR: expected a number, found '" + s + "'");
  }
}
long long Value::as_int() const {
  switch (kind) {
    case INT: return i;
    case REAL: return (long long)d;  // truncation, as int() of a float
    case BOOL: return b ? 1 : 0;
    default: throw DeckError("ERROR: expected an integer, found '" + s + "'");
  }
}
bool Value::as_bool() const {
  switch (kind) {
    case BOOL: return b;
    case INT: return i != 0;
    case REAL: return d != 0.0;
    case STR: return !s.empty();
    default: return false;
  }
}
std::string Value::as_str() const {
  std::string r;
  switch (kind) {
    case STR: r = s; break;
    case BOOL: r = b ? "TRUE" : "FALSE"; break;
    case INT: r = std::to_string(i); break;
    case REAL: {
      std::ostringstream o;
      o << d;
      r = o.str();
      break;
    }
    default: r = ""; break;
  }
  return upper(strip(r));
}

bool Namelist::has(const std::string& name) const { return vars.count(lower(name)) != 0; }

Value Namelist::get_scalar(const std::string& name, const Value& dflt) const {
  auto it = vars.find(lower(name));
  if (it == vars.end()) return dflt;
  if (it->second.is_array) {
    auto j = it->second.items.find({1});
    return j == it->second.items.end() ? dflt : j->second;
  }
  return it->second.scalar;
}

std::vector<Value> Namelist::get_array(const std::string& name, const std::vector<int>& shape,
                                       const Value& dflt) const {
  size_t total = 1;
  for (int e : shape) total *= (size_t)e;
  std::vector<Value> arr(total, dflt);
  auto it = vars.find(lower(name));
  if (it == vars.end()) return arr;
  auto put = [&](std::vector<int> idx, const Value& v) {
    while (idx.size() < shape.size()) idx.push_back(1);
    size_t off = 0;
    for (size_t d = 0; d < shape.size(); d++) {
      const int k = idx[d] - 1;
      if (k < 0 || k >= shape[d]) throw DeckError("ERROR: index out of range for " + name);
      off = off * (size_t)shape[d] + (size_t)k;
    }
    arr[off] = v;
  };
  if (!it->second.is_array) {
    put(std::vector<int>(shape.size(), 1), it->second.scalar);
  } else {
    for (const auto& kv : it->second.items) put(kv.first, kv.second);
  }
  return arr;
}

Groups parse_deck(const std::string& raw) {
  const std::string text = strip_comments(raw);
  Groups groups;
  static const std::regex grp("&(\\w+)");
  static const std::regex key_re("(\\w+)\\s*(?:\\((.*)\\))?");
  for (auto m = std::sregex_iterator(text.begin(), text.end(), grp); m != std::sregex_iterator();
       ++m) {
    const std::string name = lower((*m)[1].str());
    const size_t start = (size_t)(m->position(0) + m->length(0));
    // the group ends at the first '/' outside quotes
    char q = 0;
    size_t j = start;
    while (j < text.size()) {
      const char ch = text[j];
      if (q) {
        if (ch == q) q = 0;
      } else if (ch == '\'' || ch == '"') {
        q = ch;
      } else if (ch == '/') {
        break;
      }
      j++;
    }
    const std::string body = text.substr(start, j - start);
    Namelist nl;
    for (const auto& kv : tokens(body)) {
      std::smatch km;
      if (!std::regex_match(kv.first, km, key_re)) throw DeckError("ERROR: bad namelist item '" + kv.first + "'");
      const std::string var = lower(km[1].str());
      const bool has_sub = km[2].matched;
      std::string sub = km[2].str();
      std::vector<Value> values;
      for (const auto& it : kv.second) values.push_back(parse_value(it));
      if (!has_sub && values.size() == 1) {
        Entry e;
        e.scalar = values[0];
        nl.vars[var] = e;
        continue;
      }
      if (!has_sub) sub = ":";
      const size_t ndim = (size_t)std::count(sub.begin(), sub.end(), ',') + 1;
      const auto idx = indices(sub, extents(var, ndim));
      if (values.size() > idx.size()) throw DeckError("ERROR: too many values for " + var);
      Entry& e = nl.vars[var];
      if (!e.is_array) {
        Value old = e.scalar;
        const bool had = old.kind != Value::NONE;
        e.is_array = true;
        e.items.clear();
        if (had) e.items[{1}] = old;
      }
      for (size_t k = 0; k < values.size(); k++) e.items[idx[k]] = values[k];
    }
    groups[name] = nl;
  }
  return groups;
}

std::string read_file(const std::string& path) {
  std::ifstream f(path);
  if (!f) throw DeckError("ERROR: cannot open control file " + path);
  std::stringstream ss;
  ss << f.rdbuf();
  return ss.str();
}

bl_config build_config(const Groups& groups, int nreg, int nmat) {
  bl_config c;
  std::memset(&c, 0, sizeof c);
  static const Namelist empty;
  auto grp = [&](const char* g) -> const Namelist& {
    auto it = groups.find(g);
    return it == groups.end() ? empty : it->second;
  };
  const Namelist& ctl = grp("control");
  auto R = [](const Namelist& nl, const char* n, double d) { return nl.get_scalar(n, Value::real(d)).as_real(); };
  // time_cf_defaults (time_config.f90)
  c.time_start = R(ctl, "time_start", 0.0);
  c.time_end = R(ctl, "time_end", 1.0);
  c.dt_initial = R(ctl, "dt_initial", 1.0e-5);
  c.dt_g = R(ctl, "dt_g", 1.02);
  c.dt_min = R(ctl, "dt_min", 1.0e-8);
  c.dt_max = R(ctl, "dt_max", 1.0e-1);
  if (c.time_start > c.time_end) throw DeckError("ERROR: time_start > time_end");
  if (c.dt_min > c.dt_max) throw DeckError("ERROR: dt_min > dt_max");
  // hydro_cf_defaults (hydro_config.f90:42-77)
  c.cvisc1 = R(ctl, "cvisc1", 0.5);
  c.cvisc2 = R(ctl, "cvisc2", 0.75);
  c.cfl_sf = R(ctl, "cfl_sf", 0.5);
  c.div_sf = R(ctl, "div_sf", 0.25);
  const std::string visc = ctl.get_scalar("visc", Value::str("EDGE")).as_str();
  if (visc != "EDGE" && visc != "TENSOR") throw DeckError("ERROR: unknown value of visc");
  c.ztq = visc == "TENSOR" ? 1 : 0;
  if (c.cvisc1 < 0.0) throw DeckError("ERROR: cvisc1 < 0");
  if (c.cvisc2 < 0.0) throw DeckError("ERROR: cvisc2 < 0");
  if (c.cfl_sf < 0.0) throw DeckError("ERROR: cfl_sf < 0");
  if (c.div_sf < 0.0) throw DeckError("ERROR: div_sf < 0");
  const double kappaall = R(ctl, "kappaall", 0.0);
  const double pmeritall = R(ctl, "pmeritall", 0.0);
  const auto kreg = ctl.get_array("kappareg", {LN}, Value::real(0.0));
  const auto preg = ctl.get_array("pmeritreg", {LN}, Value::real(0.0));
  const auto zdt = ctl.get_array("zdtnotreg", {LN}, Value::boolean(false));
  const auto zml = ctl.get_array("zmidlength", {LN}, Value::boolean(false));
  if (nreg > BL_MAXREG || nmat > BL_MAXMAT) throw DeckError("ERROR: too many regions or materials");
  // setup_read.f90:239,250: MERGE(kappareg,kappaall,kappareg>0)
  for (int i = 0; i < nreg; i++) {
    const double k = kreg[i].as_real();
    c.kappareg[i] = k > 0.0 ? k : kappaall;
    const double p = preg[i].as_real();
    c.pmeritreg[i] = p > 0.0 ? p : pmeritall;
    c.zdtnotreg[i] = zdt[i].as_bool() ? 1 : 0;
    c.zmidlength[i] = zml[i].as_bool() ? 1 : 0;
  }
  // hydro_cf_rationalise (hydro_config.f90:349,368)
  c.zhg = 0;
  c.zsp = 0;
  for (int i = 0; i < nreg; i++) {
    if (c.kappareg[i] > 0.0) c.zhg = 1;
    if (c.pmeritreg[i] > 0.0) c.zsp = 1;
  }
  // global_cf_defaults / eos_cf_defaults, then CUTOFF
  const Namelist& cut = grp("cutoff");
  c.zcut = R(cut, "zcut", 1.0e-8);
  c.zerocut = R(cut, "zerocut", 1.0e-40);
  c.dencut = R(cut, "dencut", 1.0e-6);
  c.accut = R(cut, "accut", 1.0e-6);
  c.ccut = R(cut, "ccut", 1.0e-6);
  c.pcut = R(cut, "pcut", 1.0e-8);
  const char* cnames[] = {"zcut", "zerocut", "dencut", "accut", "ccut", "pcut"};
  const double cvals[] = {c.zcut, c.zerocut, c.dencut, c.accut, c.ccut, c.pcut};
  for (int k = 0; k < 6; k++)
    if (cvals[k] < 0.0) throw DeckError(std::string("ERROR: ") + cnames[k] + " < 0");
  // EOS (setup_read.f90:509-589; eos_config.f90:163-226)
  const Namelist& eos = grp("eos");
  const auto etype = eos.get_array("eos_type", {LN}, Value::str("UNKNOWN"));
  const auto eparam = eos.get_array("eos_param", {6, LN}, Value());
  c.eos_type[0] = 0;
  for (int k = 0; k < BL_NEOSPARAM; k++) c.eos_param[0][k] = 0.0;
  for (int m = 1; m <= nmat; m++) {
    const std::string t = etype[m - 1].as_str();
    int code;
    if (t == "UNKNOWN") code = -1;
    else if (t == "VOID") code = 0;
    else if (t == "IDEAL GAS") code = 1;
    else if (t == "TAIT") code = 2;
    else if (t == "JWL") code = 3;
    else throw DeckError("ERROR: unrecognised EoS type");
    c.eos_type[m] = code;
    for (int k = 0; k < 6; k++) {
      // eos_cf_defaults holds param(2,1)=-1 replicated by eos_cf_get
      // (eos_config.f90:55-58, 94-107); rows 3..6 start at zero
      const Value& v = eparam[(size_t)k * LN + (size_t)(m - 1)];
      c.eos_param[m][k] = v.kind == Value::NONE ? (k < 2 ? -1.0 : 0.0) : v.as_real();
    }
  }
  // ALE (ale_config.f90:42-49, 511-551)
  const Namelist& ale = grp("ale");
  c.ale_adv_type = (int)ale.get_scalar("adv_type", Value::integer(1)).as_int();
  c.ale_npatch = (int)ale.get_scalar("npatch", Value::integer(0)).as_int();
  c.ale_sf = R(ale, "ale_sf", 0.5);
  c.ale_zeul = ale.get_scalar("zeul", Value::boolean(false)).as_bool() ? 1 : 0;
  c.ale_zon = 0;  // no input sets ale%zon
  c.ale_mintime = DBL_MAX;
  c.ale_maxtime = DBL_MAX;
  c.ale_zexist = 0;
  if (c.ale_zeul) {
    c.ale_npatch = 1;
    c.ale_mintime = -DBL_MAX;
    c.ale_maxtime = DBL_MAX;
    c.ale_zexist = 1;
  } else if (c.ale_npatch < 0) {
    throw DeckError("ERROR: npatch < 0");
  }
  return c;
}

}  // namespace blh
