// vacgb - drop-in host program for VAC's `vac` executable on the explicit
// TVDLF/Hancock path, driving the GB300 engine through include/vacgpu.h.
//
//   vacgb [--physics=mhd|hd] [--precision=fp64|mixed] [--dump-params] < par/PROBLEM
//
// It does what `program vac` does around the time step (src/vac.t:5-157):
// reads the namelists of par/DEFAULT and then of the problem file on stdin
// (readparameters, src/vacio.t:5-531), reads the initial file
// (readfileini, binary or ascii, src/vacio.t:534-755), and runs the time
// loop with VAC's save logic (timetosave, src/vac.t:631-661): a snapshot is
// appended to filename(2) (savefileout_bin, src/vacio.t:1008-1047) and a row
// to the log filename(1) (savefilelog_default, src/vacio.t:1050-1105) at
// every save event; between save events the engine advances without host
// round trips.  Errors print the message and stop, as die() does.
//
// typeB='special' faces call the user's specialbound, which this program
// loads as a device hook (vacgpu_bound_fn) from a shared library named by
// VACGB_SPECIALBOUND=library.so:symbol.  The user's specialsource and
// getdt_special are loaded likewise from
// VACGB_SPECIALSOURCE=library.so:source_symbol[:getdt_symbol] (an empty
// source symbol installs the dt limit alone).
#include <chrono>
#include <thread>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include <dlfcn.h>

#include "../../include/vacgpu.h"

namespace {

[[noreturn]] void die(const std::string& m) {
  std::printf(" %s\n", m.c_str());
  std::exit(1);
}

std::string lower(std::string s) {
  for (auto& c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}

// ------------------------------------------------------------ namelists --
// A value list of one namelist assignment, e.g.  typeB = 8*'periodic', ...
struct Assign {
  std::string name;
  std::vector<int> idx;            // explicit subscripts (1-based), may be empty
  std::vector<std::string> vals;   // repeat counts expanded
};

struct Namelists {
  std::map<std::string, std::vector<Assign>> groups;  // group -> assignments
};

// Split a Fortran namelist stream into groups and assignments.
void parse_namelists(const std::string& text, Namelists& nl) {
  size_t i = 0, n = text.size();
  auto skip_ws = [&]() {
    while (i < n) {
      if (text[i] == '!') {
        while (i < n && text[i] != '\n') i++;
      } else if (std::isspace((unsigned char)text[i]) || text[i] == ',') {
        i++;
      } else {
        break;
      }
    }
  };
  auto read_quoted = [&]() -> std::string {
    char q = text[i++];
    std::string s;
    while (i < n) {
      if (text[i] == q) {
        if (i + 1 < n && text[i + 1] == q) {
          s += q;
          i += 2;
          continue;
        }
        i++;
        break;
      }
      s += text[i++];
    }
    return "'" + s;  // mark strings
  };
  auto read_token = [&]() -> std::string {
    skip_ws();
    if (i >= n) return "";
    if (text[i] == '\'' || text[i] == '"') return read_quoted();
    std::string s;
    int depth = 0;  // a subscript list "name(iw,iB)" keeps its commas
    while (i < n && (depth > 0 || (!std::isspace((unsigned char)text[i]) && text[i] != ',')) &&
           text[i] != '/' && text[i] != '=' && text[i] != '!') {
      if (text[i] == '*' && !s.empty()) {  // repeat count
        s += text[i++];
        if (i < n && (text[i] == '\'' || text[i] == '"')) return s + read_quoted();
        continue;
      }
      if (text[i] == '(') depth++;
      if (text[i] == ')' && depth > 0) depth--;
      if (std::isspace((unsigned char)text[i])) {
        i++;
        continue;
      }
      s += text[i++];
    }
    return s;
  };
  while (i < n) {
    skip_ws();
    if (i >= n) break;
    if (text[i] != '&' && text[i] != '$') {
      while (i < n && text[i] != '\n') i++;
      continue;
    }
    i++;
    std::string grp;
    while (i < n && !std::isspace((unsigned char)text[i])) grp += text[i++];
    grp = lower(grp);
    auto& list = nl.groups[grp];
    while (true) {
      skip_ws();
      if (i >= n) break;
      if (text[i] == '/') {
        i++;
        break;
      }
      if (text[i] == '&' || text[i] == '$') {  // &end
        while (i < n && !std::isspace((unsigned char)text[i])) i++;
        break;
      }
      std::string key;
      int kdepth = 0;  // blanks inside "name(iw, iB)" belong to the key
      while (i < n && text[i] != '=' &&
             (kdepth > 0 || !std::isspace((unsigned char)text[i]))) {
        if (text[i] == '(') kdepth++;
        if (text[i] == ')' && kdepth > 0) kdepth--;
        if (!std::isspace((unsigned char)text[i])) key += text[i];
        i++;
      }
      skip_ws();
      if (i >= n || text[i] != '=') die("Error in namelist " + grp + ": expected = after " + key);
      i++;
      Assign a;
      std::string k = lower(key);
      size_t lp = k.find('(');
      if (lp != std::string::npos) {
        std::string sub = k.substr(lp + 1, k.find(')') - lp - 1);
        std::stringstream ss(sub);
        std::string part;
        while (std::getline(ss, part, ',')) a.idx.push_back(std::atoi(part.c_str()));
        k = k.substr(0, lp);
      }
      a.name = k;
      // values until the next "name =" or "/"
      while (true) {
        skip_ws();
        if (i >= n || text[i] == '/' || text[i] == '&' || text[i] == '$') break;
        size_t save = i;
        std::string tok = read_token();
        skip_ws();
        if (i < n && text[i] == '=' && tok[0] != '\'') {  // next assignment
          i = save;
          break;
        }
        if (i < n && text[i] == '(' ) {  // name(idx)= form glued
          i = save;
          break;
        }
        size_t st = tok.find('*');
        if (st != std::string::npos && tok[0] != '\'' && st > 0 &&
            std::isdigit((unsigned char)tok[0])) {
          int rep = std::atoi(tok.substr(0, st).c_str());
          std::string v = tok.substr(st + 1);
          for (int r = 0; r < rep; r++) a.vals.push_back(v);
        } else {
          a.vals.push_back(tok);
        }
      }
      list.push_back(a);
    }
  }
}

double to_double(const std::string& v) {
  std::string s = v;
  for (auto& c : s)
    if (c == 'd' || c == 'D') c = 'e';
  return std::strtod(s.c_str(), nullptr);
}
bool to_bool(const std::string& v) {
  std::string s = lower(v);
  return s == "t" || s == ".true." || s == "true" || s == ".t.";
}
std::string to_str(const std::string& v) {
  std::string s = v.size() && v[0] == '\'' ? v.substr(1) : v;
  while (!s.empty() && s.back() == ' ') s.pop_back();
  return s;
}

// ---------------------------------------------------------------- files --
struct Snap {
  std::string head, varnames;
  int it = 0, ndim = 0, neqpar = 0, nw = 0;
  double t = 0;
  std::vector<int> nx;
  std::vector<double> eqpar, x, w;
  long long ncell() const {
    long long n = 1;
    for (int v : nx) n *= v;
    return n;
  }
};

bool read_rec(std::ifstream& f, std::vector<char>& buf) {
  int32_t n1, n2;
  if (!f.read((char*)&n1, 4)) return false;
  if (n1 < 0) die("Error in ReadFileIni: corrupt record");
  buf.resize(n1);
  if (!f.read(buf.data(), n1) || !f.read((char*)&n2, 4) || n1 != n2)
    die("Error in ReadFileIni: corrupt record");
  return true;
}

Snap read_ini_binary(const std::string& fn, int snapshot) {
  std::ifstream f(fn, std::ios::binary);
  if (!f) die("Stop: file does not exist, filenameini=" + fn);
  Snap last;
  int count = 0;
  std::vector<char> b;
  // the next record of the snapshot, at least `min` bytes (exactly, if exact)
  auto rec = [&](size_t min, bool exact, const char* what) {
    if (!read_rec(f, b)) die(std::string("Error in ReadFileIni: ") + fn + " ends before the " + what);
    if (b.size() < min || (exact && b.size() != min))
      die(std::string("Error in ReadFileIni: wrong size of the ") + what + " record in " + fn);
  };
  while (read_rec(f, b)) {
    Snap s;
    s.head = std::string(b.begin(), b.end());
    rec(24, false, "it,t,ndim,neqpar,nw");
    std::memcpy(&s.it, b.data(), 4);
    std::memcpy(&s.t, b.data() + 4, 8);
    std::memcpy(&s.ndim, b.data() + 12, 4);
    std::memcpy(&s.neqpar, b.data() + 16, 4);
    std::memcpy(&s.nw, b.data() + 20, 4);
    if (s.ndim < 0) die("Error: input file contains general grid");
    if (s.ndim < 1 || s.ndim > 3 || s.nw < 1 || s.neqpar < 0)
      die("Error in ReadFileIni: bad ndim, nw or neqpar in " + fn);
    rec(4 * (size_t)s.ndim, false, "nx");
    s.nx.resize(s.ndim);
    std::memcpy(s.nx.data(), b.data(), 4 * s.ndim);
    for (int v : s.nx)
      if (v < 1) die("Error in ReadFileIni: bad grid size in " + fn);
    rec(8 * (size_t)s.neqpar, true, "eqpar");
    s.eqpar.resize(b.size() / 8);
    std::memcpy(s.eqpar.data(), b.data(), b.size());
    rec(0, false, "varnames");
    s.varnames = std::string(b.begin(), b.end());
    const size_t bytes = 8 * (size_t)s.ncell();
    rec(bytes * s.ndim, true, "x");
    s.x.resize(b.size() / 8);
    std::memcpy(s.x.data(), b.data(), b.size());
    for (int iw = 0; iw < s.nw; iw++) {
      rec(bytes, true, "w");
      size_t o = s.w.size();
      s.w.resize(o + b.size() / 8);
      std::memcpy(s.w.data() + o, b.data(), b.size());
    }
    last = s;
    if (++count == snapshot) break;
  }
  if (!count) die("Error in ReadFileIni: empty file " + fn);
  return last;
}

Snap read_ini_ascii(const std::string& fn) {
  std::ifstream f(fn);
  if (!f) die("Stop: file does not exist, filenameini=" + fn);
  Snap s;
  std::getline(f, s.head);
  f >> s.it >> s.t >> s.ndim >> s.neqpar >> s.nw;
  // neqpar: the physics' own parameters plus the user's (nspecialpar); a
  // header asking for more than 1024 is damaged
  if (!f || s.ndim < 1 || s.ndim > 3 || s.nw < 1 || s.nw > VACGPU_MAXNW || s.neqpar < 0 ||
      s.neqpar > 1024)
    die("Error in ReadFileIni: bad header line in " + fn);
  s.nx.resize(s.ndim);
  for (auto& v : s.nx) f >> v;
  for (int v : s.nx)
    if (!f || v < 1) die("Error in ReadFileIni: bad grid size in " + fn);
  s.eqpar.resize(s.neqpar);
  for (auto& v : s.eqpar) f >> v;
  if (!f) die("Error in ReadFileIni: bad equation parameters in " + fn);
  std::string line;
  std::getline(f, line);
  std::getline(f, s.varnames);
  long long n = s.ncell();
  s.x.resize(n * s.ndim);
  s.w.resize(n * s.nw);
  for (long long c = 0; c < n; c++) {
    for (int d = 0; d < s.ndim; d++) f >> s.x[d * n + c];
    for (int iw = 0; iw < s.nw; iw++) f >> s.w[iw * n + c];
  }
  if (!f) die("Error in ReadFileIni: " + fn + " ends before its last cell");
  return s;
}

void write_rec(std::ofstream& f, const void* p, int32_t n) {
  f.write((const char*)&n, 4);
  f.write((const char*)p, n);
  f.write((const char*)&n, 4);
}

std::string pad79(std::string s) {
  s.resize(79, ' ');
  return s;
}

}  // namespace

int main(int argc, char** argv) {
  std::string physics_opt, prec_opt = "fp64";
  bool dump = false;
  for (int a = 1; a < argc; a++) {
    std::string s = argv[a];
    if (s.rfind("--physics=", 0) == 0) physics_opt = s.substr(10);
    else if (s.rfind("--precision=", 0) == 0) prec_opt = s.substr(12);
    else if (s == "--dump-params") dump = true;
    else die("usage: vacgb [--physics=mhd|hd] [--precision=fp64|mixed] [--dump-params] < par");
  }
  auto t_start = std::chrono::steady_clock::now();
  auto cputime = [&]() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
  };

  // par/DEFAULT, then the problem file on stdin (later values win)
  Namelists nl;
  {
    std::ifstream d("par/DEFAULT");
    if (d) {
      std::stringstream ss;
      ss << d.rdbuf();
      parse_namelists(ss.str(), nl);
    }
    std::stringstream ss;
    ss << std::cin.rdbuf();
    parse_namelists(ss.str(), nl);
  }
  auto find_all = [&](const std::string& name) {
    std::vector<const Assign*> out;
    for (auto& g : nl.groups)
      for (auto& a : g.second)
        if (a.name == name) out.push_back(&a);
    return out;
  };
  auto last = [&](const std::string& name) -> const Assign* {
    auto v = find_all(name);
    return v.empty() ? nullptr : v.back();
  };
  // every assignment of a 1-D array, in file order: "name = v1, v2, ..."
  // fills from element 1, "name(i) = ..." from element i; values past the
  // last element are ignored; a subscript outside 1..size, or more than one
  // subscript, stops the program
  auto fill1 = [&](const std::string& name, size_t size, auto setter) {
    for (auto* a : find_all(name)) {
      if (a->idx.size() > 1 || (!a->idx.empty() && (a->idx[0] < 1 || (size_t)a->idx[0] > size)))
        die("Error in namelist: subscript out of range for " + name);
      size_t o = a->idx.empty() ? 0 : (size_t)(a->idx[0] - 1);
      for (size_t k = 0; k < a->vals.size() && o + k < size; k++) setter(o + k, a->vals[k]);
    }
  };
  auto getd = [&](const std::string& name, double def) {
    auto a = last(name);
    return a && !a->vals.empty() ? to_double(a->vals[0]) : def;
  };
  auto geti = [&](const std::string& name, int def) {
    auto a = last(name);
    return a && !a->vals.empty() ? (int)to_double(a->vals[0]) : def;
  };
  auto getb = [&](const std::string& name, bool def) {
    auto a = last(name);
    return a && !a->vals.empty() ? to_bool(a->vals[0]) : def;
  };
  auto gets = [&](const std::string& name, const std::string& def) {
    auto a = last(name);
    return a && !a->vals.empty() ? to_str(a->vals[0]) : def;
  };

  // filelist
  std::string fini = gets("filenameini", "");
  if (fini.empty()) die("Error in ReadParameters: filenameini is not set");
  std::vector<std::string> fnames(2, "");
  fill1("filename", 2, [&](size_t k, const std::string& v) { fnames[k] = to_str(v); });
  std::string typeini = lower(gets("typefileini", "auto"));
  int snapini = geti("snapshotini", 0);
  if (getb("fullgridini", false) || getb("fullgridout", false))
    die("fullgridini/fullgridout=T are not on this path");
  if (typeini == "auto") {
    std::ifstream f(fini, std::ios::binary);
    if (!f) die("Stop: file does not exist, filenameini=" + fini);
    unsigned char h[91] = {0};
    f.read((char*)h, 91);
    if (h[0] && h[1] && h[2] && h[3]) typeini = "ascii";
    else if (!h[88] && !h[89] && (h[87] == 24 || h[90] == 24)) typeini = "binary";
    else die("Error in VAC: Unknown typefileini=special");
  }
  Snap ini = typeini == "ascii" ? read_ini_ascii(fini) : read_ini_binary(fini, snapini);
  std::string typeout = lower(gets("typefileout", "auto"));
  if (typeout == "auto") typeout = typeini;
  if (typeout != "binary") die("typefileout=" + typeout + ": this host writes binary .out files");

  // physics from the header suffix _mhdNN/_hdNN (setheaderstrings)
  std::string phys = physics_opt;
  int ndir = ini.ndim;
  size_t us = ini.head.rfind('_');
  if (phys.empty() && us != std::string::npos) {
    std::string suf = ini.head.substr(us + 1);
    while (!suf.empty() && suf.back() == ' ') suf.pop_back();
    if (suf.rfind("mhd", 0) == 0) phys = "mhd";
    else if (suf.rfind("hd", 0) == 0) phys = "hd";
    size_t p = suf.find_first_of("0123456789");
    if (p != std::string::npos && p + 1 < suf.size()) ndir = suf[p + 1] - '0';
  }
  if (phys.empty()) die("physics unknown: give --physics=mhd or --physics=hd");
  // the header's ndir digit: a vector has ndim..3 components
  if (ndir < ini.ndim || ndir > 3)
    die("Error in ReadFileIni: header " + ini.head + " gives ndir outside ndim..3");
  const int physics = phys == "mhd" ? VACGPU_PHYS_MHD : VACGPU_PHYS_HD;
  const int nw = physics == VACGPU_PHYS_MHD ? 2 + 2 * ndir : 2 + ndir;
  if (ini.nw != nw || nw > VACGPU_MAXNW) die("Incompatible number of variables in " + fini);

  vacgpu_params p;
  vacgpu_default_params(&p, ini.ndim, ndir, physics, ini.nx.data());
  p.precision = prec_opt == "mixed" ? VACGPU_PREC_MIXED : VACGPU_PREC_FP64;
  for (size_t k = 0; k < ini.eqpar.size() && k < VACGPU_MAXEQPAR; k++) p.eqpar[k] = ini.eqpar[k];
  fill1("eqpar", VACGPU_MAXEQPAR,
        [&](size_t k, const std::string& v) { p.eqpar[k] = to_double(v); });

  // methodlist (readparameters' harmonisation, src/vacio.t:216-364)
  std::vector<std::string> typefull(nw, "tvdlf"), typelim(nw, "minmod");
  fill1("typefull", nw, [&](size_t k, const std::string& v) { typefull[k] = lower(to_str(v)); });
  fill1("typelimiter", nw, [&](size_t k, const std::string& v) { typelim[k] = lower(to_str(v)); });
  std::string tf1 = "nul";
  for (auto& t : typefull)
    if (t != "nul") tf1 = t;
  if (tf1 == "tvdlf") p.typefull = VACGPU_TVDLF;
  else if (tf1 == "tvdlf1") p.typefull = VACGPU_TVDLF1;
  else if (tf1 == "tvdmu") p.typefull = VACGPU_TVDMU;
  else if (tf1 == "tvdmu1") p.typefull = VACGPU_TVDMU1;
  else die("Error in Advect1: " + tf1 +
           " is not on this path (tvdlf, tvdlf1, tvdmu, tvdmu1)");
  // typeentropy, entropycoef (per characteristic wave) and divbwave of the
  // Roe dissipation (src/vacio.t:35,80; par/DEFAULT:47)
  const char* entnames[] = {"nul", "harten", "powell", "ratio", "yee"};
  fill1("typeentropy", nw, [&](size_t k, const std::string& v) {
    std::string t = lower(to_str(v));
    int e = -1;
    for (int m = 0; m < 5; m++)
      if (t == entnames[m]) e = m;
    if (e < 0) die("No such type of entropy fix:" + t);
    p.typeentropy[k] = e;
  });
  fill1("entropycoef", nw, [&](size_t k, const std::string& v) { p.entropycoef[k] = to_double(v); });
  p.divbwave = getb("divbwave", true);
  const char* limnames[] = {"minmod", "woodward", "superbee", "vanleer", "albada"};
  for (int iw = 0; iw < nw; iw++) {
    int l = -1;
    for (int k = 0; k < 5; k++)
      if (typelim[iw] == limnames[k]) l = k;
    if (l < 0) die("Error in dwLimiter: No such TVD limiter:" + typelim[iw]);
    p.typelimiter[iw] = l;
  }
  if (gets("typeadvance", "twostep") != "twostep")
    die("typeadvance=" + gets("typeadvance", "") + " is not on this path");
  p.useprimitive = getb("useprimitive", false);
  p.compactres = getb("compactres", false);
  if (getb("sourcesplit", false)) die("sourcesplit=T is not on this path");
  std::string tds = lower(gets("typedimsplit", "default"));
  bool dimsplit = getb("dimsplit", true);
  if (tds == "default") tds = dimsplit ? "xyyx" : "unsplit";
  p.dimsplit = tds != "unsplit";
  p.typedimsplit = tds == "xy" ? VACGPU_SPLIT_XY : VACGPU_SPLIT_XYYX;
  std::string tl = lower(gets("typelimited", "original"));
  if (!p.dimsplit && tl == "original") tl = "previous";
  p.typelimited = tl == "previous" ? VACGPU_LIMITED_PREVIOUS
                  : tl == "predictor" ? VACGPU_LIMITED_PREDICTOR
                                      : VACGPU_LIMITED_ORIGINAL;
  p.divbfix = getb("divbfix", true);
  p.sourceunsplit = getb("sourceunsplit", true);
  p.smallp = getd("smallp", -1.0);
  p.smallpcoeff = getd("smallpcoeff", 1.0e-6);
  p.smallfix = getb("smallfix", false);
  p.smallrho = getd("smallrho", -1.0);
  p.smallrhocoeff = getd("smallrhocoeff", 1.0e-6);
  p.vacuumrho = getd("vacuumrho", -1.0);
  // paramlist, stoplist
  p.courantpar = getd("courantpar", 0.8);
  p.dtpar = getd("dtpar", -1.0);
  p.dtdiffpar = getd("dtdiffpar", 0.5);
  p.slowsteps = geti("slowsteps", 0);
  p.dtcantgrow = getb("dtcantgrow", false);
  p.itmax = geti("itmax", 1000000);
  p.tmax = getd("tmax", 1e99);
  p.tmaxexact = getb("tmaxexact", false);
  p.dtmin = getd("dtmin", 1e-99);
  // boundlist: typeB(iw,iB) in column order (iw fastest), default 'cont'
  const char* bcnames[] = {"cont", "periodic", "symm", "asymm", "fixed",
                           "fixed1", "cont1", "grad1", "symm0", "special"};
  for (auto* a : find_all("typeb")) {
    size_t o = 0;
    // typeB(iw,iB): iw in 1..nw, iB in 1..2*ndim; typeB(q) in 1..nw*2*ndim
    const size_t nb = (size_t)nw * 2 * ini.ndim;
    bool bad = a->idx.size() > 2;
    for (size_t m = 0; m < a->idx.size(); m++) bad = bad || a->idx[m] < 1;
    if (a->idx.size() == 2)
      bad = bad || a->idx[0] > nw || a->idx[1] > 2 * ini.ndim;
    else if (a->idx.size() == 1)
      bad = bad || (size_t)a->idx[0] > nb;
    if (bad) die("Error in namelist: subscript out of range for typeB");
    if (a->idx.size() == 2) o = (a->idx[1] - 1) * nw + (a->idx[0] - 1);
    else if (a->idx.size() == 1) o = a->idx[0] - 1;
    for (size_t k = 0; k < a->vals.size(); k++) {
      size_t q = o + k;
      int ib = (int)(q / nw), iw = (int)(q % nw);
      if (ib >= 2 * ini.ndim) break;
      std::string t = lower(to_str(a->vals[k]));
      int b = -1;
      for (int m = 0; m < 10; m++)
        if (t == bcnames[m]) b = m;
      if (b < 0) die("Error in GetBoundary: boundary type " + t + " is not on this path");
      p.typeB[ib][iw] = b;
    }
  }
  // savelist: tsave(isave,ifile), itsave(isave,ifile), dtsave(ifile), ditsave(ifile)
  const int NSAVE = 100;
  // one sentinel past the last save slot, where the save counters stop
  double tsave[2][NSAVE + 1];
  int itsave[2][NSAVE + 1];
  double dtsave[2] = {1e99, 1e99};
  int ditsave[2] = {10000000, 10000000};
  for (int f = 0; f < 2; f++)
    for (int k = 0; k <= NSAVE; k++) {
      tsave[f][k] = 1e99;
      itsave[f][k] = 10000000;
    }
  auto fill2 = [&](const char* nm, auto setter) {
    for (auto* a : find_all(nm)) {
      size_t o = 0;
      // name(isave,ifile): isave in 1..NSAVE, ifile in 1..2; name(q) in 1..2*NSAVE
      bool bad = a->idx.size() > 2;
      for (size_t m = 0; m < a->idx.size(); m++) bad = bad || a->idx[m] < 1;
      if (a->idx.size() == 2)
        bad = bad || a->idx[0] > NSAVE || a->idx[1] > 2;
      else if (a->idx.size() == 1)
        bad = bad || a->idx[0] > 2 * NSAVE;
      if (bad) die(std::string("Error in namelist: subscript out of range for ") + nm);
      if (a->idx.size() == 2) o = (a->idx[1] - 1) * NSAVE + (a->idx[0] - 1);
      else if (a->idx.size() == 1) o = a->idx[0] - 1;
      for (size_t k = 0; k < a->vals.size(); k++) setter(o + k, a->vals[k]);
    }
  };
  fill2("tsave", [&](size_t q, const std::string& v) {
    if (q < 2 * NSAVE) tsave[q / NSAVE][q % NSAVE] = to_double(v);
  });
  fill2("itsave", [&](size_t q, const std::string& v) {
    if (q < 2 * NSAVE) itsave[q / NSAVE][q % NSAVE] = (int)to_double(v);
  });
  fill1("dtsave", 2, [&](size_t k, const std::string& v) { dtsave[k] = to_double(v); });
  fill1("ditsave", 2, [&](size_t k, const std::string& v) { ditsave[k] = (int)to_double(v); });

  if (dump) {
    std::printf("{\"ndim\": %d, \"ndir\": %d, \"physics\": %d, \"nw\": %d, \"nx\": [%d, %d, %d],"
                " \"gamma\": %.17g, \"typefull\": %d, \"typelimiter\": [",
                p.ndim, p.ndir, p.physics, p.nw, p.nx[0], p.nx[1], p.nx[2], p.eqpar[0], p.typefull);
    for (int iw = 0; iw < nw; iw++) std::printf("%s%d", iw ? ", " : "", p.typelimiter[iw]);
    std::printf("], \"typelimited\": %d, \"dimsplit\": %d, \"typedimsplit\": %d, \"divbfix\": %d,"
                " \"courantpar\": %.17g, \"dtpar\": %.17g, \"itmax\": %d, \"tmax\": %.17g,"
                " \"useprimitive\": %d, \"smallfix\": %d, \"smallp\": %.17g, \"smallrho\": %.17g,"
                " \"smallrhocoeff\": %.17g, \"vacuumrho\": %.17g, \"typeB\": [",
                p.typelimited, p.dimsplit, p.typedimsplit, p.divbfix, p.courantpar, p.dtpar,
                p.itmax, p.tmax, p.useprimitive, p.smallfix, p.smallp, p.smallrho, p.smallrhocoeff,
                p.vacuumrho);
    for (int ib = 0; ib < 2 * p.ndim; ib++) {
      std::printf("%s[", ib ? ", " : "");
      for (int iw = 0; iw < nw; iw++) std::printf("%s%d", iw ? ", " : "", p.typeB[ib][iw]);
      std::printf("]");
    }
    std::printf("], \"typeentropy\": [");
    for (int il = 0; il < nw; il++) std::printf("%s%d", il ? ", " : "", p.typeentropy[il]);
    std::printf("], \"entropycoef\": [");
    for (int il = 0; il < nw; il++) std::printf("%s%.17g", il ? ", " : "", p.entropycoef[il]);
    std::printf("], \"divbwave\": %d, \"eqpar\": [%.17g, %.17g]", p.divbwave, p.eqpar[0],
                p.eqpar[1]);
    std::printf(", \"ditsave\": [%d, %d], \"dtsave\": [%.17g, %.17g], \"itsave1\": [%d, %d],"
                " \"tsave2\": [%.17g, %.17g], \"filenames\": [\"%s\", \"%s\"]}\n",
                ditsave[0], ditsave[1], dtsave[0], dtsave[1], itsave[0][0], itsave[0][1],
                tsave[1][0], tsave[1][1], fnames[0].c_str(), fnames[1].c_str());
    return 0;
  }

  vacgpu_handle* h = nullptr;
  auto chk = [&](int rc) {
    if (rc) {
      char buf[1024];
      vacgpu_last_error(buf, sizeof buf);
      die(buf);
    }
  };
  chk(vacgpu_create(&p, &h));
  bool special = false;
  for (int ib = 0; ib < 2 * p.ndim; ib++)
    for (int iw = 0; iw < nw; iw++) special |= p.typeB[ib][iw] == VACGPU_BC_SPECIAL;
  if (special) {
    // the user's specialbound as a device hook: VACGB_SPECIALBOUND=lib.so:symbol
    const char* spec = std::getenv("VACGB_SPECIALBOUND");
    if (!spec) die("Special boundary is not defined (set VACGB_SPECIALBOUND=lib.so:symbol)");
    std::string sp(spec);
    size_t colon = sp.rfind(':');
    if (colon == std::string::npos) die("VACGB_SPECIALBOUND must be library.so:symbol");
    void* lib = dlopen(sp.substr(0, colon).c_str(), RTLD_NOW | RTLD_LOCAL);
    if (!lib) die(std::string("VACGB_SPECIALBOUND: ") + dlerror());
    void* fn = dlsym(lib, sp.substr(colon + 1).c_str());
    if (!fn) die("VACGB_SPECIALBOUND: no symbol " + sp.substr(colon + 1));
    chk(vacgpu_register_bound(h, (vacgpu_bound_fn)fn, nullptr));
  }
  if (const char* spec = std::getenv("VACGB_SPECIALSOURCE")) {
    // library.so:source_symbol[:getdt_symbol]
    std::string sp(spec);
    size_t c1 = sp.find(".so:");
    if (c1 == std::string::npos)
      die("VACGB_SPECIALSOURCE must be library.so:source_symbol[:getdt_symbol]");
    c1 += 3;
    void* lib = dlopen(sp.substr(0, c1).c_str(), RTLD_NOW | RTLD_LOCAL);
    if (!lib) die(std::string("VACGB_SPECIALSOURCE: ") + dlerror());
    std::string rest = sp.substr(c1 + 1);
    size_t c2 = rest.find(':');
    std::string ssym = rest.substr(0, c2);
    std::string dsym = c2 == std::string::npos ? "" : rest.substr(c2 + 1);
    void* fs = ssym.empty() ? nullptr : dlsym(lib, ssym.c_str());
    void* fd = dsym.empty() ? nullptr : dlsym(lib, dsym.c_str());
    if (!ssym.empty() && !fs) die("VACGB_SPECIALSOURCE: no symbol " + ssym);
    if (!dsym.empty() && !fd) die("VACGB_SPECIALSOURCE: no symbol " + dsym);
    chk(vacgpu_register_source_fn(h, (vacgpu_source_fn)fs, (vacgpu_dtspecial_fn)fd, nullptr));
  }
  chk(vacgpu_set_grid(h, ini.x.data()));
  chk(vacgpu_upload(h, ini.w.data(), ini.it, ini.t));
  std::printf("Start Advance  %10.3f sec\n", cputime());

  int it = ini.it;
  double t = ini.t, dt = 0.0;
  int isavet[2] = {0, 0}, isaveit[2] = {0, 0}, itsavelast[2] = {it, it};
  double tsavelast[2] = {t, t};
  std::ofstream outf, logf;
  std::vector<double> wbuf(ini.w.size());
  std::string headout = ini.head;
  // savefileout_bin's records of one snapshot (state w taken at sit, st_)
  auto write_out = [&](int sit, double st_, const double* w) {
    write_rec(outf, pad79(headout).data(), 79);
    char rec2[24];
    int32_t ndimout = p.ndim, neq = (int32_t)ini.eqpar.size(), nww = nw;
    std::memcpy(rec2, &sit, 4);
    std::memcpy(rec2 + 4, &st_, 8);
    std::memcpy(rec2 + 12, &ndimout, 4);
    std::memcpy(rec2 + 16, &neq, 4);
    std::memcpy(rec2 + 20, &nww, 4);
    write_rec(outf, rec2, 24);
    write_rec(outf, ini.nx.data(), 4 * p.ndim);
    std::vector<double> eq(ini.eqpar.size());
    for (size_t k = 0; k < eq.size(); k++) eq[k] = k < VACGPU_MAXEQPAR ? p.eqpar[k] : ini.eqpar[k];
    write_rec(outf, eq.data(), (int32_t)(8 * eq.size()));
    write_rec(outf, pad79(ini.varnames).data(), 79);
    write_rec(outf, ini.x.data(), (int32_t)(8 * ini.x.size()));
    const long long n = ini.ncell();
    for (int iw = 0; iw < nw; iw++) write_rec(outf, w + iw * n, (int32_t)(8 * n));
    outf.flush();
  };
  // A save event of the .out file takes a snapshot (vacgpu_snapshot_begin)
  // and hands it to a writer thread, which waits for the copy and writes the
  // records while the next steps run; the next event, and the end of the
  // run, join it first, so records stay in order.  VACGB_SYNC_SAVE=1 writes
  // each record before the run continues (vacgpu_download).
  const bool sync_save = std::getenv("VACGB_SYNC_SAVE") && std::atoi(std::getenv("VACGB_SYNC_SAVE"));
  std::thread writer;
  std::string writer_err;
  auto join_writer = [&]() {
    if (writer.joinable()) writer.join();
    if (!writer_err.empty()) die(writer_err);
  };
  auto savefile = [&](int ifile) {
    if (ifile == 1) {  // savefileout_bin
      if (fnames[1].empty()) return;
      join_writer();
      if (!outf.is_open()) outf.open(fnames[1], std::ios::binary);
      if (sync_save) {
        chk(vacgpu_download(h, wbuf.data()));
        write_out(it, t, wbuf.data());
        return;
      }
      chk(vacgpu_snapshot_begin(h, 0));
      const int sit = it;
      const double st_ = t;
      writer = std::thread([&, sit, st_]() {
        // the records go out straight from the library's page-locked copy
        const double* snapw = nullptr;
        if (vacgpu_snapshot_wait(h, 0, nullptr) == 0) snapw = vacgpu_snapshot_data(h, 0);
        if (!snapw) {
          char buf[1024];
          vacgpu_last_error(buf, sizeof buf);
          writer_err = buf;
          return;
        }
        write_out(sit, st_, snapw);
      });
    } else {  // savefilelog_default
      if (fnames[0].empty()) return;
      if (!logf.is_open()) {
        logf.open(fnames[0]);
        logf << headout << "\n" << "it   t   dt    " << ini.varnames << "\n";
      }
      std::vector<double> wm(nw);
      chk(vacgpu_sums(h, wm.data()));
      char line[64];
      std::snprintf(line, sizeof line, "%7d", it);
      logf << line;
      std::vector<double> vals = {t, dt};
      vals.insert(vals.end(), wm.begin(), wm.end());
      for (double v : vals) {
        std::snprintf(line, sizeof line, "%13.5E", v);
        logf << line;
      }
      logf << "\n";
      logf.flush();
    }
  };
  // timetosave, src/vac.t:631-661
  auto timetosave = [&](int f) {
    bool ok = false;
    if (t >= tsave[f][isavet[f]]) {
      ok = true;
      if (isavet[f] < NSAVE) isavet[f]++;
    }
    if (it == itsave[f][isaveit[f]]) {
      ok = true;
      if (isaveit[f] < NSAVE) isaveit[f]++;
    }
    if (it == itsavelast[f] + ditsave[f]) ok = true;
    if (t >= tsavelast[f] + dtsave[f]) ok = true;
    if (ok) {
      tsavelast[f] = t;
      itsavelast[f] = it;
    }
    return ok;
  };
  while (true) {
    for (int f = 0; f < 2; f++)
      if (timetosave(f)) savefile(f);
    // next save event: steps and time
    long long next_it = 1LL << 40;
    double next_t = 1e300;
    for (int f = 0; f < 2; f++) {
      next_it = std::min<long long>(next_it, (long long)itsave[f][isaveit[f]] - it);
      next_it = std::min<long long>(next_it, (long long)itsavelast[f] + ditsave[f] - it);
      next_t = std::min(next_t, tsave[f][isavet[f]]);
      next_t = std::min(next_t, tsavelast[f] + dtsave[f]);
    }
    int maxsteps = (int)std::max<long long>(1, std::min<long long>(next_it, 1 << 30));
    int fin = 0;
    chk(vacgpu_step(h, maxsteps, next_t, &t, &it, &dt, &fin));
    if (fin) break;
  }
  const double tfin = cputime();
  for (int f = 0; f < 2; f++)
    if (itsavelast[f] < it) savefile(f);
  join_writer();
  std::printf("Finish Advance %10.3f sec\n", tfin);
  int nerror[4];
  chk(vacgpu_error_counts(h, nerror));
  const char* desc[] = {"Pressure below psmall", "Density below rhosmall",
                        "Courant number above 1", "Poisson solver failed"};
  for (int k = 0; k < 4; k++)
    if (nerror[k] > 0) {
      std::printf("Error (code=%2d) occurred %5d times !!!\n", k + 1, nerror[k]);
      std::printf("Error description: %s\n", desc[k]);
    }
  vacgpu_destroy(h);
  std::printf("Finished VAC   %10.3f sec\n", cputime());
  return 0;
}
