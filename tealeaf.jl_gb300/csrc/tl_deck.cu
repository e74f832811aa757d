// tl_deck.cu -- the tea.in reader inside the library: Settings(infile)
// (src/settings.jl:90-135) and readstate (src/settings.jl:142-173), host code.
//
// Lines are stripped of surrounding whitespace.  A line that starts with
// "state" is a state; "use_<name>" picks the solver; lines that start with
// '*' or hold no '=' are skipped.  Otherwise the key is the text before the
// first '=' with every '_' removed (then stripped), the value the text between
// the first and the second '='; `initial_timestep` is an alias of dtinit.
// Unknown keys and values that do not parse are skipped with a warning, as
// the reference warns.  dx and dy are computed from the domain once the whole
// deck is read (settings.jl:132-133).  A state's bounds are inset by dx/100
// (dy/100): in reference mode with dx, dy as they stand when the state line is
// read (the default 10 unless the deck set dx itself, settings.jl:159-162), in
// tealeaf mode with the deck's final dx, dy.  A malformed state line is an
// error, as it throws in the reference.
#include <cerrno>
#include <climits>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/tealeaf_gb300.h"

namespace {

struct RawState {
  double density = 0, energy = 0, xmin = 0, ymin = 0, xmax = 0, ymax = 0, radius = 0;
  int geometry = TL_GEOM_RECTANGULAR;
  int given = 0;            // which bounds the line set (1 xmin, 2 ymin, 4 xmax, 8 ymax)
  double pdx = 10, pdy = 10;  // dx, dy when the line was read
};

std::string strip(const std::string &s) {
  size_t a = 0, b = s.size();
  while (a < b && (s[a] == ' ' || s[a] == '\t' || s[a] == '\r' || s[a] == '\n' || s[a] == '\v' || s[a] == '\f')) ++a;
  while (b > a && (s[b - 1] == ' ' || s[b - 1] == '\t' || s[b - 1] == '\r' || s[b - 1] == '\n' || s[b - 1] == '\v' ||
                   s[b - 1] == '\f'))
    --b;
  return s.substr(a, b - a);
}

std::vector<std::string> split(const std::string &s, char sep) {
  std::vector<std::string> out;
  size_t a = 0;
  for (;;) {
    const size_t b = s.find(sep, a);
    if (b == std::string::npos) {
      out.push_back(s.substr(a));
      return out;
    }
    out.push_back(s.substr(a, b - a));
    a = b + 1;
  }
}

// An optionally signed run of decimal digits.
bool parse_int(const std::string &v, long long *out) {
  const std::string t = strip(v);
  size_t i = (!t.empty() && (t[0] == '+' || t[0] == '-')) ? 1 : 0;
  if (i >= t.size()) return false;
  for (size_t k = i; k < t.size(); ++k)
    if (t[k] < '0' || t[k] > '9') return false;
  errno = 0;
  const long long x = strtoll(t.c_str(), nullptr, 10);
  if (errno == ERANGE) return false;
  *out = x;
  return true;
}

bool parse_bool(const std::string &v, int *out) {
  const std::string t = strip(v);
  if (t == "true" || t == "1") {
    *out = 1;
    return true;
  }
  if (t == "false" || t == "0") {
    *out = 0;
    return true;
  }
  return false;
}

bool parse_f64(const std::string &v, double *out) {
  const std::string t = strip(v);
  if (t.empty()) return false;
  char *end = nullptr;
  const double x = strtod(t.c_str(), &end);
  if (end != t.c_str() + t.size()) return false;
  *out = x;
  return true;
}

bool set_int(int *dst, const std::string &v) {
  long long x;
  if (!parse_int(v, &x) || x < INT_MIN || x > INT_MAX) return false;
  *dst = (int)x;
  return true;
}

int fail(char *err, int errlen, const char *fmt, ...) {
  if (err && errlen > 0) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(err, (size_t)errlen, fmt, ap);
    va_end(ap);
  }
  return TL_ERR_ARG;
}

}  // namespace

extern "C" int tl_parse_deck(const char *text, int mode, tl_deck *deck, tl_state *states, int maxstates, char *err,
                             int errlen) {
  if (!text || !deck || (maxstates > 0 && !states) || (mode != TL_MODE_REFERENCE && mode != TL_MODE_TEALEAF))
    return fail(err, errlen, "tl_parse_deck: invalid argument");
  if (err && errlen > 0) err[0] = '\0';
  // Settings() defaults (src/settings.jl:39-78)
  tl_deck d;
  memset(&d, 0, sizeof d);
  d.endstep = LLONG_MAX;
  d.presteps = 30;
  d.maxiters = 10000;
  d.coefficient = TL_CONDUCTIVITY;
  d.ppcginnersteps = 10;
  d.summaryfrequency = 10;
  d.halodepth = 2;
  d.errorswitch = 0;
  d.checkresult = 1;
  d.eps = 1e-15;
  d.dtinit = 0.1;
  d.endtime = 10.0;
  d.epslim = 1e-5;
  d.solver = TL_SOLVER_CG;
  d.xcells = 10;
  d.ycells = 10;
  d.xmin = 0.0;
  d.ymin = 0.0;
  d.xmax = 100.0;
  d.ymax = 100.0;
  d.dx = 10.0;
  d.dy = 10.0;
  std::vector<RawState> raw;
  const std::vector<std::string> lines = split(std::string(text), '\n');
  for (size_t ln = 0; ln < lines.size(); ++ln) {
    const std::string line = strip(lines[ln]);
    if (line.compare(0, 5, "state") == 0) {  // readstate (settings.jl:142-173)
      const std::vector<std::string> pieces = split(line, ' ');
      long long num = 0;
      if (pieces.size() < 2 || !parse_int(pieces[1], &num))
        return fail(err, errlen, "line %zu: state number does not parse (src/settings.jl:146)", ln + 1);
      RawState st;
      st.pdx = d.dx;
      st.pdy = d.dy;
      for (size_t k = 2; k < pieces.size(); ++k) {
        const std::vector<std::string> kv = split(pieces[k], '=');
        if (kv.size() < 2)
          return fail(err, errlen, "line %zu: state item '%s' has no '=' (src/settings.jl:148)", ln + 1,
                      pieces[k].c_str());
        const std::string &key = kv[0], &val = kv[1];
        double x = 0;
        if (key == "density" || key == "energy") {
          if (!parse_f64(val, &x)) return fail(err, errlen, "line %zu: %s does not parse", ln + 1, key.c_str());
          (key == "density" ? st.density : st.energy) = x;
        }
        if (num == 1) continue;  // state 1 is the background (settings.jl:152-154)
        if (key == "xmin" || key == "ymin" || key == "xmax" || key == "ymax") {
          if (!parse_f64(val, &x)) return fail(err, errlen, "line %zu: %s does not parse", ln + 1, key.c_str());
          if (key == "xmin") st.xmin = x, st.given |= 1;
          else if (key == "ymin") st.ymin = x, st.given |= 2;
          else if (key == "xmax") st.xmax = x, st.given |= 4;
          else st.ymax = x, st.given |= 8;
        } else if (key == "radius") {
          if (!parse_f64(val, &x)) return fail(err, errlen, "line %zu: radius does not parse", ln + 1);
          st.radius = x;
        } else if (key == "geometry") {
          if (val == "rectangle") st.geometry = TL_GEOM_RECTANGULAR;
          else if (val == "circular") st.geometry = TL_GEOM_CIRCULAR;
          else if (val == "point") st.geometry = TL_GEOM_POINT;
          else return fail(err, errlen, "line %zu: unknown geometry '%s'", ln + 1, val.c_str());
        }
      }
      raw.push_back(st);
      continue;
    }
    if (line.compare(0, 4, "use_") == 0) {  // settings.jl:103-111
      const std::string name = line.substr(4);
      if (name == "cg") d.solver = TL_SOLVER_CG;
      else if (name == "ppcg") d.solver = TL_SOLVER_PPCG;
      else if (name == "cheby") d.solver = TL_SOLVER_CHEBY;
      else if (name == "jacobi") d.solver = TL_SOLVER_JACOBI;
      else ++d.warnings;
      continue;
    }
    if (line.empty() || line[0] == '*' || line.find('=') == std::string::npos) continue;
    const std::vector<std::string> parts = split(line, '=');
    std::string key;
    for (char ch : parts[0])
      if (ch != '_') key += ch;
    key = strip(key);
    const std::string &val = parts[1];
    if (key == "initialtimestep") key = "dtinit";
    bool ok = true;
    if (key == "endstep") {
      long long x;
      ok = parse_int(val, &x);
      if (ok) d.endstep = x;
    } else if (key == "presteps") ok = set_int(&d.presteps, val);
    else if (key == "maxiters") ok = set_int(&d.maxiters, val);
    else if (key == "coefficient") ok = set_int(&d.coefficient, val);
    else if (key == "ppcginnersteps") ok = set_int(&d.ppcginnersteps, val);
    else if (key == "summaryfrequency") ok = set_int(&d.summaryfrequency, val);
    else if (key == "halodepth") ok = set_int(&d.halodepth, val);
    else if (key == "xcells") ok = set_int(&d.xcells, val);
    else if (key == "ycells") ok = set_int(&d.ycells, val);
    else if (key == "errorswitch") ok = parse_bool(val, &d.errorswitch);
    else if (key == "checkresult") ok = parse_bool(val, &d.checkresult);
    else if (key == "eps") ok = parse_f64(val, &d.eps);
    else if (key == "dtinit") ok = parse_f64(val, &d.dtinit);
    else if (key == "endtime") ok = parse_f64(val, &d.endtime);
    else if (key == "epslim") ok = parse_f64(val, &d.epslim);
    else if (key == "xmin") ok = parse_f64(val, &d.xmin);
    else if (key == "ymin") ok = parse_f64(val, &d.ymin);
    else if (key == "xmax") ok = parse_f64(val, &d.xmax);
    else if (key == "ymax") ok = parse_f64(val, &d.ymax);
    else if (key == "dx") ok = parse_f64(val, &d.dx);
    else if (key == "dy") ok = parse_f64(val, &d.dy);
    else ok = false;
    if (!ok) ++d.warnings;
  }
  d.dx = (d.xmax - d.xmin) / d.xcells;  // settings.jl:132-133
  d.dy = (d.ymax - d.ymin) / d.ycells;
  d.nstates = (int)raw.size();
  for (int k = 0; k < d.nstates && k < maxstates; ++k) {
    const RawState &r = raw[k];
    const double ix = mode == TL_MODE_REFERENCE ? r.pdx : d.dx, iy = mode == TL_MODE_REFERENCE ? r.pdy : d.dy;
    tl_state s;
    s.density = r.density;
    s.energy = r.energy;
    s.xmin = (r.given & 1) ? r.xmin + ix / 100 : r.xmin;
    s.ymin = (r.given & 2) ? r.ymin + iy / 100 : r.ymin;
    s.xmax = (r.given & 4) ? r.xmax - ix / 100 : r.xmax;
    s.ymax = (r.given & 8) ? r.ymax - iy / 100 : r.ymax;
    s.radius = r.radius;
    s.geometry = r.geometry;
    states[k] = s;
  }
  *deck = d;
  return TL_OK;
}
