// rl_host.cpp -- readers for the reference's input files, ray family, per-line tables and
// the spectrum writer. Formats (RADLITE/ of pontoppi/radlite):
//   radlite.inp        main.F:488-686 (format >= 100), setup.F:1117-1137 (setup -551),
//                      comment lines stripped and records cut at 16 characters (tools.F:6-20)
//   radius.inp         grid.F:716-727 + ghost nodes grid.F:782-789
//   theta.inp          grid.F:1103-1176 (mirror about the equator, ghost nodes)
//   density.inp        setup.F:1453-1500 via read_scalar_field setup.F:1584-1690
//   velocity.inp       setup.F:754-789          turbulence.inp setup.F:803-850
//   abundance.inp      setup.F:864-919          dustdens.inp   setup.F:681-746, 525-670
//   dusttemp.info/_final.dat setup.F:159-235, 295-420
//   dustopac.inp, dustopac_N.inp dust.F:92-447  frequency.inp  grid.F:1427-1482
//   starinfo.inp       star.F:543-569           starspectrum.inp / starspec.inp star.F:449-537
//   interstellfield.inp star.F:690-727 (outer boundary 3)
//   scatsource.dat     source.F:494-543         line.inp header line.F:142-200, 3918-3935
//   linespectrum.inp   telescope.F:86-257       moldata.dat    line.F:1826-1985 (fixed columns)
//   levelpop.info + levelpop_<mol>.dat line.F:811-950
// Output: linespectrum_<mol>.dat as header_line_spectrum/write_line_spectrum
// (telescope.F:1662-1804).
#include "rl_host.h"

#include <sys/stat.h>
#include <unistd.h>

#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>

namespace rl {
namespace {

struct Fail {
  std::string msg;
};
[[noreturn]] void fail(const std::string& m) { throw Fail{m}; }

// Every input file a parse opens or probes, with its size and modification time: the key
// of the binary input cache.
struct InputStamp {
  std::string name;
  long long size = -1, mtime_ns = 0;   // size -1: absent
};
thread_local std::vector<InputStamp>* g_stamps = nullptr;

InputStamp stat_input(const std::string& dir, const std::string& name) {
  InputStamp s;
  s.name = name;
  struct stat st;
  if (::stat((dir + "/" + name).c_str(), &st) == 0) {
    s.size = (long long)st.st_size;
    s.mtime_ns = (long long)st.st_mtim.tv_sec * 1000000000LL + (long long)st.st_mtim.tv_nsec;
  }
  return s;
}

void stamp(const std::string& dir, const std::string& name) {
  if (g_stamps) g_stamps->push_back(stat_input(dir, name));
}

// Record-oriented reader with Fortran list-directed semantics: each read statement
// starts on a new record, consumes tokens across records as needed and drops the
// remainder of its last record. Tokens are views into the file buffer and numbers are
// parsed with from_chars (correctly rounded, like strtod), without allocations.
class Records {
 public:
  Records(const std::string& dir, const std::string& name) : name_(name) {
    stamp(dir, name);
    std::ifstream f(dir + "/" + name, std::ios::binary);
    if (!f) fail("cannot open " + dir + "/" + name);
    f.seekg(0, std::ios::end);
    const std::streamoff n = f.tellg();
    f.seekg(0, std::ios::beg);
    buf_.resize(n > 0 ? (size_t)n : 0);
    if (n > 0) f.read(&buf_[0], n);
  }
  struct FromText {};
  Records(FromText, std::string text, std::string name) : name_(std::move(name)), buf_(std::move(text)) {}
  // next record as [b, e) without the line end; false at the end of the file
  bool view(const char*& b, const char*& e) {
    if (pos_ >= buf_.size()) return false;
    const char* base = buf_.data();
    const void* nl = std::memchr(base + pos_, '\n', buf_.size() - pos_);
    const size_t end = nl ? (size_t)((const char*)nl - base) : buf_.size();
    b = base + pos_;
    e = base + end;
    if (e > b && e[-1] == '\r') e--;
    pos_ = end + 1;
    return true;
  }
  bool line(std::string& out) {
    const char *b, *e;
    if (!view(b, e)) return false;
    out.assign(b, e);
    return true;
  }
  struct Tok { const char* p; size_t n; };
  void list(size_t n, std::vector<Tok>& toks) {
    toks.clear();
    const char *b, *e;
    while (toks.size() < n) {
      if (!view(b, e)) fail(name_ + ": unexpected end of file");
      const char* i = b;
      while (i < e && toks.size() < n) {
        while (i < e && (*i == ' ' || *i == '\t' || *i == ',')) i++;
        if (i >= e) break;
        const char* j = i;
        while (j < e && *j != ' ' && *j != '\t' && *j != ',') j++;
        toks.push_back(Tok{i, (size_t)(j - i)});
        i = j;
      }
    }
  }
  double num(const Tok& t) {
    char tmp[64];
    const char* b = t.p;
    const char* e = t.p + t.n;
    // Fortran D exponents and a leading '+' go through a small copy
    bool copy = t.n < sizeof tmp && (*b == '+' || std::memchr(b, 'd', t.n) || std::memchr(b, 'D', t.n));
    if (copy) {
      size_t k = 0;
      for (const char* c = (*b == '+' ? b + 1 : b); c < e; c++) tmp[k++] = (*c == 'd' || *c == 'D') ? 'e' : *c;
      b = tmp;
      e = tmp + k;
    }
    double v = 0.0;
    const auto r = std::from_chars(b, e, v);
    if (r.ec == std::errc::invalid_argument || r.ptr == b) fail(name_ + ": not a number: '" + std::string(t.p, t.n) + "'");
    if (r.ec == std::errc::result_out_of_range) {   // overflow and underflow as strtod gives them
      const std::string z(b, r.ptr);
      v = std::strtod(z.c_str(), nullptr);
    }
    const char* q = r.ptr;
    if (q < e && (*q == '+' || *q == '-')) {   // Fortran exponent without a letter, e.g. 1.0+05
      long ex = 0;
      const auto r2 = std::from_chars(q + 1, e, ex);
      if (r2.ec == std::errc() && r2.ptr == e && r2.ptr != q + 1) return v * std::pow(10.0, (double)(*q == '-' ? -ex : ex));
    }
    if (q != e) fail(name_ + ": not a number: '" + std::string(t.p, t.n) + "'");
    return v;
  }
  double d() { list(1, t_); return num(t_[0]); }
  int i() { return (int)d(); }
  std::string s() { list(1, t_); return std::string(t_[0].p, t_[0].n); }
  void dn(size_t n, double* out) {
    list(n, t_);
    for (size_t k = 0; k < n; k++) out[k] = num(t_[k]);
  }
  std::vector<double> head(size_t n) {
    std::vector<double> v(n);
    dn(n, v.data());
    return v;
  }
  const std::string& name() const { return name_; }

 private:
  std::string name_, buf_;
  size_t pos_ = 0;
  std::vector<Tok> t_;
};

bool exists(const std::string& dir, const std::string& name) {
  stamp(dir, name);
  std::ifstream f(dir + "/" + name);
  return (bool)f;
}

// Fortran fixed-column numeric field (Iw, Fw.d, Ew.d input; blanks ignored).
double col(const std::string& line, size_t start, size_t width, int d) {
  std::string b;
  bool dot = false;
  for (size_t i = start; i < start + width && i < line.size(); i++) {
    char c = line[i];
    if (c == ' ' || c == '\t') continue;
    if (c == 'd' || c == 'D') c = 'e';
    if (c == '.') dot = true;
    b.push_back(c);
  }
  if (b.empty()) return 0.0;
  if (dot || d == 0) return std::strtod(b.c_str(), nullptr);
  size_t e = b.find_first_of("eE");
  if (e == std::string::npos) {
    for (size_t k = 1; k < b.size(); k++) if (b[k] == '+' || b[k] == '-') { e = k; break; }
  }
  if (e == std::string::npos) return std::strtod(b.c_str(), nullptr) * std::pow(10.0, -d);
  const double mant = std::strtod(b.substr(0, e).c_str(), nullptr);
  const double ex = std::strtod(b.substr(e + ((b[e] == 'e' || b[e] == 'E') ? 1 : 0)).c_str(), nullptr);
  return mant * std::pow(10.0, ex - d);
}


void read_scalar(const std::string& dir, const std::string& name, const Model& m, std::vector<double>& out) {
  Records f(dir, name);
  const auto h = f.head(3);
  if ((int)h[2] == 0) fail(name + ": theta mirroring flag must be 1");
  if ((int)h[0] != m.nr || 2 * (int)h[1] != m.ny) fail(name + ": inconsistent dimensions");
  out.resize(m.ncell());
  for (int c = 0; c < m.ncell(); c++) out[c] = f.d();
}

void read_radlite_inp(const std::string& dir, Model& m) {
  Records raw(dir, "radlite.inp");
  std::string text, l;
  while (raw.line(l)) {
    if (!l.empty() && (l[0] == '#' || l[0] == ';' || l[0] == '%' || l[0] == '=')) continue;
    if (l.size() > 16) l.resize(16);
    text += l;
    text += '\n';
  }
  Records f(Records::FromText{}, text, "radlite.inp");
  const int fmt = f.i();
  if (fmt < 100) fail("radlite.inp: input format " + std::to_string(fmt) + " not supported");
  f.i(); f.i();
  if (fmt >= 103) f.i();
  f.d(); f.i(); f.i();
  for (int k = 0; k < 6; k++) f.d();
  m.outer_bc = f.i();
  f.i();   // inner boundary: forced to 2 (star in vacuum) by setup -551
  f.i();
  f.d();   // default inclination: replaced by linespectrum.inp
  m.nphi = f.i();
  m.dbdr = f.i();
  m.nrext = f.i();
  for (int k = 0; k < 4; k++) f.i();
  if (fmt >= 101) f.i();
  if (fmt >= 102) f.i();
  f.i();
  if (fmt >= 104) f.i();
  const int wp = f.i();
  if (wp != -551) fail("radlite.inp: setup type " + std::to_string(wp) + " not supported");
  const int dodust = f.i(), doline = f.i();
  m.line_dust = f.i();
  m.starpump = f.i();
  if (dodust != 0 || doline == 0) fail("radlite.inp: only line transfer (dust 0, lines 1) is supported");
  if (m.nrext == 0) fail("radlite.inp: nrrayextra must be non-zero");
  if (m.outer_bc != 0 && m.outer_bc != 2 && m.outer_bc != 3)
    fail("radlite.inp: outer boundary type " + std::to_string(m.outer_bc) + " not supported");
}

void read_grid(const std::string& dir, Model& m) {
  {
    Records f(dir, "radius.inp");
    m.nr = f.i();
    if (m.nr < 3) fail("radius.inp: need at least 3 radii");
    m.R.assign(m.nr + 4, 0.0);
    for (int ix = 1; ix <= m.nr; ix++) m.R[ix + 1] = f.d();
  }
  auto R = [&](int ix) -> double& { return m.R[ix + 1]; };
  const int nr = m.nr;
  R(0) = R(1) * R(1) / R(2);
  R(-1) = R(0) * R(0) / R(1);
  R(nr + 1) = R(nr) * R(nr) / R(nr - 1);
  R(nr + 2) = R(nr + 1) * R(nr + 1) / R(nr);
  for (int ix = 1; ix < nr; ix++) {
    if (!(R(ix + 1) > R(ix))) fail("radius.inp: radii must increase");
    if (R(ix + 1) / R(ix) - 1.0 < 1.0e4 * 1.0e-10) fail("radius.inp: radial grid too fine for the telescope safety number");
  }
  {
    Records f(dir, "theta.inp");
    const auto h = f.head(2);
    m.nth = (int)h[0];
    if ((int)h[1] == 0) fail("theta.inp: theta mirroring flag must be 1");
    if (m.nth < 2) fail("theta.inp: need at least 2 points");
    m.ny = 2 * m.nth;
    m.TH.assign(m.ny + 4, 0.0);
    for (int iy = 1; iy <= m.nth; iy++) {
      const double t = f.d();
      if (t > 1.5707963268 || t < 0.0) fail("theta.inp: theta outside [0, pi/2]");
      m.TH[iy + 1] = t;
    }
  }
  auto T = [&](int iy) -> double& { return m.TH[iy + 1]; };
  const int ny = m.ny;
  for (int iy = 1; iy <= m.nth; iy++) T(2 * m.nth + 1 - iy) = 3.14159265359 - T(iy);
  T(0) = -T(1);
  T(-1) = -T(2);
  // the reference uses the single-precision constant 2*3.1415926e0 here
  const double twopi_f = (double)(2.0f * 3.1415926f);
  T(ny + 1) = twopi_f - T(ny);
  T(ny + 2) = twopi_f - T(ny - 1);
}

void read_dust(const std::string& dir, Model& m) {
  const int ncell = m.ncell();
  {
    const std::string dn = exists(dir, "dustdensity.inp") ? "dustdensity.inp" : "dustdens.inp";
    Records f(dir, dn);
    const auto h = f.head(4);
    m.nspec = (int)h[0];
    if (m.nspec < 1 || m.nspec > 4) fail(dn + ": 1 to 4 dust species supported");
    if ((int)h[1] != m.nr || 2 * (int)h[2] != m.ny || (int)h[3] == 0) fail(dn + ": inconsistent dimensions");
    m.drho.resize((size_t)m.nspec * ncell);
    for (auto& v : m.drho) v = f.d();
  }
  {
    Records info(dir, "dusttemp.info");
    const int flnr = info.i();
    const std::string fn = flnr == -2 ? std::string("dusttemp_final.dat") : "dusttemp_" + std::to_string(flnr) + ".dat";
    Records f(dir, fn);
    const auto h = f.head(4);
    if ((int)h[0] != m.nspec || (int)h[1] != m.nr || 2 * (int)h[2] != m.ny) fail(fn + ": inconsistent dimensions");
    m.nsize.assign(m.nspec, 1);
    m.dtemp.assign((size_t)m.nspec * 4 * ncell, 0.0);
    for (int s = 0; s < m.nspec; s++) {
      const int nsz = f.i();
      if (nsz < 1 || nsz > 4) fail(fn + ": 1 to 4 grain sizes supported");
      m.nsize[s] = nsz;
      for (int z = 0; z < nsz; z++)
        for (int c = 0; c < ncell; c++) m.dtemp[((size_t)s * 4 + z) * ncell + c] = f.d();
    }
  }
  {
    Records f(dir, "dustopac.inp");
    const int fmt = f.i();
    const int nsp = f.i();
    f.s();
    if (nsp != m.nspec) fail("dustopac.inp: species count differs from the dust density");
    m.kabs.assign((size_t)m.nspec * 4 * m.ncont, 0.0);
    m.ksca.assign((size_t)m.nspec * 4 * m.ncont, 0.0);
    for (int s = 0; s < nsp; s++) {
      const int mode = f.i();
      if (fmt >= 2) {
        const int q = f.i();
        if (q == 2) f.d();
        else if (q == 3) { f.d(); f.d(); }
      }
      const int ifile = f.i();
      if (mode == -2) { f.d(); f.d(); }
      else if (mode == -3) { f.d(); f.d(); f.d(); f.d(); }
      else if (mode != -1) fail("dustopac.inp: read mode " + std::to_string(mode) + " not supported");
      const std::string fn = "dustopac_" + std::to_string(ifile) + ".inp";
      Records g(dir, fn);
      const auto h = g.head(2);
      // "-1 nfreq" then "nsize idum ntemp": tables for ntemp temperature ranges, each
      // preceded by its range (read_dustopac_file, dust.F:320-480; the reference is built
      // with DUST_OPAC_TEMPDEP). The line dust reads the first table only (line.F:3582-3605).
      int nfreq = (int)h[0], nsz = (int)h[1], ntemp = 1;
      const bool trange = nfreq == -1;
      if (trange) {
        nfreq = nsz;
        const auto h2 = g.head(3);
        nsz = (int)h2[0];
        ntemp = (int)h2[2];
        if (ntemp < 1) fail(fn + ": temperature range count must be positive");
      }
      if (nfreq != m.ncont) fail(fn + ": frequency count differs from frequency.inp");
      if (nsz != m.nsize[s]) fail(fn + ": grain size count differs from the dust temperatures");
      double bold = 0.0;
      for (int t = 0; t < ntemp; t++) {
        if (trange) {
          const auto ab = g.head(2);
          const double a = ab[0], b = ab[1];
          if (a < bold) fail(fn + ": temperature ranges overlap");
          if (std::fabs((a - bold) / (a + bold)) > 1.0e-3) fail(fn + ": gap between temperature ranges");
          if (a < 0.0 || b < 0.0 || b < a) fail(fn + ": invalid temperature range");
          bold = b;
        }
        for (int i = 0; i < m.ncont; i++)
          for (int z = 0; z < nsz; z++) {
            const double v = g.d();
            if (t == 0) m.kabs[((size_t)s * 4 + z) * m.ncont + i] = v;
          }
        for (int i = 0; i < m.ncont; i++)
          for (int z = 0; z < nsz; z++) {
            const double v = g.d();
            if (t == 0) m.ksca[((size_t)s * 4 + z) * m.ncont + i] = v;
          }
      }
      f.s();
    }
  }
  if (exists(dir, "scatsource.dat")) {
    Records f(dir, "scatsource.dat");
    f.head(4);
    m.scat.assign((size_t)m.ncont * ncell, 0.0);
    for (int i = 0; i < m.ncont; i++)
      for (int it = 1; it <= m.nth; it++)
        for (int ir = 1; ir <= m.nr; ir++) m.scat[(size_t)i * ncell + (ir - 1) * m.nth + (it - 1)] += f.d();
  }
}

void read_gas(const std::string& dir, Model& m) {
  const int ncell = m.ncell();
  read_scalar(dir, "density.inp", m, m.rho);
  if (!exists(dir, "abundance.inp")) fail("abundance.inp is required");
  {
    Records f(dir, "abundance.inp");
    const auto h = f.head(2);
    if ((int)h[0] != m.nr || (int)h[1] != m.nth) fail("abundance.inp: inconsistent dimensions");
    m.abun.resize(ncell);
    double two[2];
    for (int c = 0; c < ncell; c++) { f.dn(2, two); m.abun[c] = two[0]; }
  }
  m.vel.assign((size_t)3 * ncell, 0.0);
  if (exists(dir, "velocity.inp")) {
    Records f(dir, "velocity.inp");
    const auto h = f.head(2);
    if ((int)h[0] != m.nr || (int)h[1] != m.nth) fail("velocity.inp: inconsistent dimensions");
    for (int c = 0; c < ncell; c++) f.dn(3, &m.vel[3 * (size_t)c]);
  }
  if (!exists(dir, "turbulence.inp")) fail("turbulence.inp is required (local line width)");
  {
    Records f(dir, "turbulence.inp");
    f.i();
    const auto h = f.head(2);
    if ((int)h[0] != m.nr || (int)h[1] != m.nth) fail("turbulence.inp: inconsistent dimensions");
    m.lw.resize(ncell);
    for (int c = 0; c < ncell; c++) m.lw[c] = f.d();
  }
}

void read_linespectrum(const std::string& dir, Model& m) {
  Records f(dir, "linespectrum.inp");
  const int fmt = f.i();
  m.style = 0;
  if (fmt == 1) m.style = f.i();
  if (fmt < 0 || fmt > 1) fail("linespectrum.inp: format " + std::to_string(fmt) + " unknown");
  f.s();
  if (f.i() != 2) fail("linespectrum.inp: telescope format must be 2");
  f.s();
  m.vmax = f.d();
  m.dv = f.d();
  f.s();
  if (f.i() != 2) fail("linespectrum.inp: object format must be 2");
  std::string mf = f.s();
  const size_t p = mf.find(".dat");
  if (p == std::string::npos) fail("linespectrum.inp: molecule file name must end with .dat");
  m.molfile = mf.substr(0, p + 4);
  m.molname = mf.substr(0, p);
  const int cmd = f.i();
  if (cmd == 1) fail("linespectrum.inp: command 1 is not implemented in the reference either");
  if (cmd != 0 && cmd != 2) fail("linespectrum.inp: command " + std::to_string(cmd) + " unknown");
  m.command = cmd;
  f.d();   // distance: the spectrum is computed at 1 pc (main.F:206,213)
  m.incl_rad = f.d() * 0.0174532925199;
  m.radvelo = f.d();
  m.nlspec = f.i();
  m.ilstart = f.i();
  if (cmd == 2) {   // position-velocity cube (telescope.F:190-218)
    PVSpec& pv = m.pv;
    pv.nx = f.i();
    pv.ny = f.i();
    const int sizespec = f.i();
    pv.szimx = f.d();
    pv.szimy = f.d();
    pv.phioff = f.d();
    pv.xoff = f.d();
    pv.yoff = f.d();
    pv.addstar = f.i();
    // 0 (arcsec) draws a warning in the reference, which then reads the sizes as for 1 (cm)
    if (sizespec != 0 && sizespec != 1) fail("linespectrum.inp: size specifier " + std::to_string(sizespec) + " unknown");
    pv.sizespec = sizespec;
  }
}

void read_molecule(const std::string& dir, Model& m) {
  Records f(dir, m.molfile);
  std::string l;
  f.s(); f.s(); f.s();
  if (!f.line(l)) fail("moldata: end of file");   // (F4.1) molecular weight
  f.s();
  if (!f.line(l)) fail("moldata: end of file");
  const int nlev = (int)col(l, 0, 6, 0);
  if (nlev < 2) fail("moldata: need at least 2 levels");
  f.s();
  m.Ecm.resize(nlev);
  m.gdeg.resize(nlev);
  for (int i = 0; i < nlev; i++) {
    if (!f.line(l)) fail("moldata: end of file in the level list");
    m.Ecm[i] = col(l, 5, 12, 4);
    m.gdeg[i] = col(l, 17, 7, 1);
  }
  f.s();
  if (!f.line(l)) fail("moldata: end of file");
  const int nlin = (int)col(l, 0, 6, 0);
  if (nlin < 1) fail("moldata: need at least 1 line");
  f.s();
  m.lup.resize(nlin); m.ldn.resize(nlin); m.Aud.resize(nlin); m.lfreq.resize(nlin);
  for (int i = 0; i < nlin; i++) {
    if (!f.line(l)) fail("moldata: end of file in the line list");
    m.lup[i] = (int)col(l, 5, 5, 0);
    m.ldn[i] = (int)col(l, 10, 5, 0);
    m.Aud[i] = col(l, 15, 12, 3);
  }
  for (int i = 0; i < nlin; i++) {
    if (m.lup[i] < 1 || m.ldn[i] < 1 || m.lup[i] > nlev || m.ldn[i] > nlev || m.lup[i] <= m.ldn[i])
      fail("moldata: line " + std::to_string(i + 1) + " has invalid levels");
    m.lfreq[i] = 1.509160e26 * (1.986468498e-16 * m.Ecm[m.lup[i] - 1] - 1.986468498e-16 * m.Ecm[m.ldn[i] - 1]);
    if (!(m.lfreq[i] > 0.0)) fail("moldata: line " + std::to_string(i + 1) + " has a non-positive frequency");
  }
  if (m.ilstart < 1 || m.ilstart + m.nlspec - 1 > nlin || m.nlspec < 1)
    fail("linespectrum.inp: spectrum of a non-existing line requested");
  // the run then starts at line 1 whatever the file asked (main.F:204); the check above
  // still uses the requested start (telescope.F:292-299)
  m.ilstart = 1;
}

void read_levelpop(const std::string& dir, Model& m) {
  Records info(dir, "levelpop.info");
  const int fnr = info.i();
  if (fnr == -3) {   // line.F:847-870: the second record must name a levelpop_*.dat file
    const std::string nm = info.s();
    if (nm.compare(0, 9, "levelpop_") != 0 || nm.find(".dat", 9) == std::string::npos)
      fail("levelpop.info: expected a levelpop_<name>.dat file name, got '" + nm + "'");
  }
  std::string fn;
  if (fnr == -1) fn = "levelpop.dat";
  else if (fnr == -2) fn = "levelpop_final.dat";
  else if (fnr == -3) fn = "levelpop_" + m.molname + ".dat";
  else fn = "levelpop_" + std::to_string(fnr) + ".dat";
  Records f(dir, fn);
  const auto h = f.head(4);
  if ((int)h[0] != m.nr || (int)h[1] != m.nth || (int)h[3] != 1) fail(fn + ": inconsistent dimensions");
  m.nlev = (int)h[2];
  if (m.nlev < 2) fail(fn + ": need at least 2 levels");
  std::vector<double> tmp(m.nlev);
  f.dn(m.nlev, tmp.data());
  f.dn(m.nlev, tmp.data());
  m.pop.resize((size_t)m.ncell() * m.nlev);
  for (int c = 0; c < m.ncell(); c++) f.dn(m.nlev, &m.pop[(size_t)c * m.nlev]);
  for (size_t i = 0; i < m.lup.size(); i++)
    if (m.lup[i] > m.nlev || m.ldn[i] > m.nlev) fail(fn + ": fewer levels than line " + std::to_string(i + 1) + " needs");
}

void read_star(const std::string& dir, Model& m) {
  if (exists(dir, "starinfo.inp")) {
    Records f(dir, "starinfo.inp");
    f.i();
    m.rstar = f.d();
  } else {
    m.rstar = m.R[2] * 1.0e-3;
  }
  m.starcont.assign(m.ncont, 0.0);
  if (m.starpump == 0) return;
  if (exists(dir, "starspec.inp") && exists(dir, "starspectrum.inp"))
    fail("both starspec.inp and starspectrum.inp present");
  if (exists(dir, "starspec.inp")) {
    Records f(dir, "starspec.inp");
    if (f.i() != m.ncont) fail("starspec.inp: frequency count differs from frequency.inp");
    for (int i = 0; i < m.ncont; i++) m.starcont[i] = f.d();
  } else {
    Records f(dir, "starspectrum.inp");
    if (f.i() != m.ncont) fail("starspectrum.inp: frequency count differs from frequency.inp");
    double two[2];
    for (int i = 0; i < m.ncont; i++) {
      f.dn(2, two);
      if (std::fabs(two[0] - m.cnu[i]) / (two[0] + m.cnu[i]) > 1.0e-3) fail("starspectrum.inp: frequencies differ from frequency.inp");
      m.starcont[i] = 3.0308410e36 * two[1] / (m.rstar * m.rstar);
    }
  }
}

}  // namespace

double bplanck(double temp, double nu) {   // setup.F:937-952
  if (temp == 0.0) return 0.0;
  return 1.47455e-47 * nu * nu * nu / (std::exp(4.7989e-11 * nu / temp) - 1.0) + 1.0e-290;
}

// bracketing by bisection: j with xx[j-1] < x <= xx[j] in 1-based terms
int bracket(const std::vector<double>& xx, double x) {
  const int n = (int)xx.size();
  const bool asc = xx[n - 1] > xx[0];
  int lo = 0, hi = n + 1;
  while (hi - lo != 1) {
    const int m = (hi + lo) / 2;
    if ((x > xx[m - 1]) == asc) lo = m; else hi = m;
  }
  return lo;
}

// interstellfield.inp, the outer boundary of type 3 (read_interstellfield, star.F:690-727):
// the count of frequency.inp, then one intensity per frequency
static void read_isrf(const std::string& dir, Model& m) {
  if (stat_input(dir, "interstellfield.inp").size < 0)
    fail("radlite.inp: outer boundary type 3 needs the file interstellfield.inp");
  Records f(dir, "interstellfield.inp");
  if (f.i() != m.ncont) fail("interstellfield.inp: frequency count differs from frequency.inp");
  m.isrf.resize(m.ncont);
  for (auto& v : m.isrf) v = f.d();
}

void finish_model(Model& m) {
  m.aksmax = 0.0;
  for (double v : m.lw) if (v > m.aksmax) m.aksmax = v;
  m.nfr = (int)(2.0 * m.vmax / m.dv + 1);
  m.vmax = 0.5 * (m.nfr - 1) * m.dv;
}

static int parse_dir(const std::string& dir, Model& m, std::string& err) {
  try {
    read_radlite_inp(dir, m);
    read_grid(dir, m);
    {
      Records f(dir, "frequency.inp");
      m.ncont = f.i();
      if (m.ncont < 2) fail("frequency.inp: need at least 2 frequencies");
      m.cnu.resize(m.ncont);
      for (auto& v : m.cnu) v = f.d();
    }
    if (m.outer_bc == 3) read_isrf(dir, m);
    {
      Records f(dir, "line.inp");
      const int fmt = f.i();
      if (fmt == 2) f.i();
      else if (fmt != 1) fail("line.inp: format " + std::to_string(fmt) + " unknown");
      m.umass = f.d();
    }
    if (m.line_dust) read_dust(dir, m);
    read_gas(dir, m);
    read_linespectrum(dir, m);
    read_molecule(dir, m);
    read_levelpop(dir, m);
    read_star(dir, m);
    finish_model(m);
    if (m.nfr < 2) fail("passband needs at least 2 channels");
    if (m.style != 1) fail("linespectrum.inp: only output style 1 (F_nu) is supported");
  } catch (const Fail& f) {
    err = f.msg;
    return -1;
  }
  return 0;
}

namespace {

// Every member of Model, in one order, for the cache writer, reader and checksum.
template <typename V>
void visit_model(Model& m, V& v) {
  v(m.nr); v(m.nth); v(m.ny); v(m.R); v(m.TH); v(m.rho); v(m.abun); v(m.lw); v(m.vel);
  v(m.nspec); v(m.nsize); v(m.drho); v(m.dtemp); v(m.ncont); v(m.cnu); v(m.kabs); v(m.ksca); v(m.scat);
  v(m.nlev); v(m.pop); v(m.molname); v(m.molfile); v(m.Ecm); v(m.gdeg); v(m.lup); v(m.ldn); v(m.Aud); v(m.lfreq);
  v(m.umass); v(m.rstar); v(m.starcont); v(m.starpump); v(m.outer_bc); v(m.line_dust); v(m.incl_rad); v(m.nphi);
  v(m.dbdr); v(m.nrext); v(m.vmax); v(m.dv); v(m.radvelo); v(m.nlspec); v(m.ilstart); v(m.style); v(m.nfr);
  v(m.command); v(m.pv.nx); v(m.pv.ny); v(m.pv.szimx); v(m.pv.szimy); v(m.pv.phioff); v(m.pv.xoff); v(m.pv.yoff);
  v(m.pv.addstar); v(m.pv.sizespec); v(m.aksmax); v(m.isrf);
}

struct Writer {
  std::string out;
  void raw(const void* p, size_t n) { out.append(static_cast<const char*>(p), n); }
  void operator()(int& x) { raw(&x, sizeof x); }
  void operator()(long long& x) { raw(&x, sizeof x); }
  void operator()(double& x) { raw(&x, sizeof x); }
  void operator()(std::string& x) { long long n = (long long)x.size(); raw(&n, sizeof n); raw(x.data(), x.size()); }
  template <typename T> void operator()(std::vector<T>& x) {
    long long n = (long long)x.size();
    raw(&n, sizeof n);
    if (n) raw(x.data(), sizeof(T) * x.size());
  }
};

struct Reader {
  const char* p;
  const char* e;
  bool ok = true;
  void raw(void* d, size_t n) {
    if (!ok || (size_t)(e - p) < n) { ok = false; return; }
    std::memcpy(d, p, n);
    p += n;
  }
  long long count() {
    long long n = 0;
    raw(&n, sizeof n);
    if (n < 0 || n > (long long)(e - p)) { ok = false; n = 0; }
    return n;
  }
  void operator()(int& x) { raw(&x, sizeof x); }
  void operator()(long long& x) { raw(&x, sizeof x); }
  void operator()(double& x) { raw(&x, sizeof x); }
  void operator()(std::string& x) { const long long n = count(); x.assign(ok ? p : "", ok ? (size_t)n : 0); if (ok) p += n; }
  template <typename T> void operator()(std::vector<T>& x) {
    const long long n = count();
    if (!ok || (size_t)n * sizeof(T) > (size_t)(e - p)) { ok = false; return; }
    x.resize((size_t)n);
    raw(x.data(), sizeof(T) * (size_t)n);
  }
};

// 64-bit FNV-1a over bytes (cache file names and the model checksum)
struct Hasher {
  unsigned long long h = 1469598103934665603ULL;
  void raw(const void* p, size_t n) {
    const unsigned char* b = static_cast<const unsigned char*>(p);
    for (size_t i = 0; i < n; i++) { h ^= b[i]; h *= 1099511628211ULL; }
  }
  void operator()(int& x) { raw(&x, sizeof x); }
  void operator()(double& x) { raw(&x, sizeof x); }
  void operator()(std::string& x) { raw(x.data(), x.size()); raw("\0", 1); }
  template <typename T> void operator()(std::vector<T>& x) {
    const long long n = (long long)x.size();
    raw(&n, sizeof n);
    if (n) raw(x.data(), sizeof(T) * x.size());
  }
};

constexpr char kCacheMagic[8] = {'R', 'L', 'G', 'P', 'U', 'I', 'N', '4'};

std::string cache_path(const std::string& cache_dir, const std::string& key) {
  Hasher h;
  std::string k = key;
  h(k);
  char b[32];
  std::snprintf(b, sizeof b, "%016llx.rlin", h.h);
  return cache_dir + "/" + b;
}

std::string real_dir(const std::string& dir) {
  char buf[4096];
  return ::realpath(dir.c_str(), buf) ? std::string(buf) : dir;
}

// The cached model of `dir` if every input it was parsed from is unchanged.
bool load_cached(const std::string& cache_dir, const std::string& dir, Model& m) {
  const std::string key = real_dir(dir);
  std::ifstream f(cache_path(cache_dir, key), std::ios::binary);
  if (!f) return false;
  f.seekg(0, std::ios::end);
  const std::streamoff n = f.tellg();
  f.seekg(0, std::ios::beg);
  if (n <= 0) return false;
  std::string buf((size_t)n, '\0');
  if (!f.read(&buf[0], n)) return false;
  if (buf.size() < sizeof kCacheMagic || std::memcmp(buf.data(), kCacheMagic, sizeof kCacheMagic) != 0) return false;
  Reader r{buf.data() + sizeof kCacheMagic, buf.data() + buf.size()};
  std::string kdir;
  r(kdir);
  if (!r.ok || kdir != key) return false;
  long long ns = 0;
  r(ns);
  if (!r.ok || ns < 0 || ns > 4096) return false;
  for (long long i = 0; i < ns; i++) {
    InputStamp s;
    r(s.name); r(s.size); r(s.mtime_ns);
    if (!r.ok) return false;
    const InputStamp now = stat_input(dir, s.name);
    if (now.size != s.size || now.mtime_ns != s.mtime_ns) return false;
  }
  Model c;
  visit_model(c, r);
  if (!r.ok || r.p != r.e) return false;
  m = std::move(c);
  return true;
}

void save_cached(const std::string& cache_dir, const std::string& dir, Model& m, std::vector<InputStamp>& stamps) {
  Writer w;
  w.raw(kCacheMagic, sizeof kCacheMagic);
  std::string key = real_dir(dir);
  w(key);
  long long ns = (long long)stamps.size();
  w(ns);
  for (auto& s : stamps) { w(s.name); w(s.size); w(s.mtime_ns); }
  visit_model(m, w);
  const std::string path = cache_path(cache_dir, key);
  const std::string tmp = path + "." + std::to_string((long long)::getpid()) + ".tmp";
  FILE* fp = std::fopen(tmp.c_str(), "wb");
  if (!fp) return;   // the cache is an optimisation: a failure to write it is not an error
  const bool ok = std::fwrite(w.out.data(), 1, w.out.size(), fp) == w.out.size();
  if (std::fclose(fp) == 0 && ok) std::rename(tmp.c_str(), path.c_str());
  else std::remove(tmp.c_str());
}

}  // namespace

// Parse the input files of `dir`. With RLGPU_INPUT_CACHE set to a writable directory,
// the parsed model is also kept there in binary, keyed by the directory's real path and
// by the size and modification time of every input file the parse opened or probed; a
// later load of an unchanged directory reads the binary instead of the text.
int load_dir(const std::string& dir, Model& m, std::string& err) {
  const char* cdir = std::getenv("RLGPU_INPUT_CACHE");
  const bool cache = cdir && *cdir;
  if (cache && load_cached(cdir, dir, m)) return 0;
  std::vector<InputStamp> stamps;
  g_stamps = cache ? &stamps : nullptr;
  const int rc = parse_dir(dir, m, err);
  g_stamps = nullptr;
  if (rc == 0 && cache) save_cached(cdir, dir, m, stamps);
  return rc;
}

unsigned long long model_checksum(const Model& m) {
  Hasher h;
  Model& mm = const_cast<Model&>(m);
  visit_model(mm, h);
  return h.h;
}

int setup_camera(const Model& m, double incl, int nphi, int dbdr, int nrext, Camera& cam, std::string& err) {
  if (nphi < 1) { err = "camera: nphi must be positive"; return -1; }
  if (dbdr < 1) { err = "camera: dbdr must be positive"; return -1; }
  if (nrext == 0) { err = "camera: nrrayextra must be non-zero"; return -1; }
  if (incl == 0.0) { err = "camera: inclination 0 is not supported (the reference divides by it)"; return -1; }
  if (std::fabs(incl) < 1.0e-1) incl = (double)0.1f * std::fabs(incl) / incl;
  const double rstar = m.rstar, R1 = m.R[2];
  if (rstar > R1) { err = "camera: star larger than the inner grid radius"; return -1; }
  const int nrrextra = std::abs(nrext), nrref = 10;
  cam.incl_rad = incl;
  cam.theta0 = incl + 1.0e-4;
  cam.nphi = nphi;
  const double sinth0 = std::sin(cam.theta0);
  const double dphi = 6.28318530718 / (1.0 * nphi);
  double phi = 0.5 * dphi;
  std::vector<double> zh(nphi), xh(nphi);
  for (int k = 0; k < nphi; k++) {
    zh[k] = -std::sin(phi) / sinth0;
    double dum = 1.0 - zh[k] * zh[k] * sinth0 * sinth0;
    dum = dum + 1.0e2 * 1.0e-10;
    if (dum < 0.0) { err = "camera: negative discriminant in the ray setup"; return -1; }
    xh[k] = std::cos(phi) > 0.0 ? std::sqrt(dum) : -std::sqrt(dum);
    phi = phi + dphi;
  }
  cam.nrr = nrrextra + nrref + dbdr * (m.nr - 1);
  cam.nrays = 1 + cam.nrr * nphi;
  cam.x0.assign(cam.nrays, 0.0);
  cam.z0.assign(cam.nrays, 0.0);
  cam.rays_r.assign(cam.nrr + 1, 0.0);
  cam.ri.assign(cam.nrr + 2, 0.0);
  int iray = 1, irad = 1;
  auto ring = [&](double rc) {
    cam.rays_r[irad++] = rc;
    for (int k = 0; k < nphi; k++) { cam.x0[iray] = rc * xh[k]; cam.z0[iray] = rc * zh[k]; iray++; }
  };
  double ref1 = 0.5, ref2 = 0.0;
  for (int ix = 1; ix <= nrrextra + nrref; ix++) {
    if (ix <= nrrextra) ring(((ix - 1) * (R1 - rstar) / nrrextra) + rstar);
    else {
      ref2 = ref2 + ref1;
      ref1 = ref1 / 2;
      ring(((nrrextra + ref2) * (R1 - rstar) / (nrrextra + 1.0)) + rstar);
    }
  }
  for (int ix = 1; ix <= m.nr - 1; ix++) {
    const double Rx = m.R[ix + 1], Rn = m.R[ix + 2];
    ring(Rx * (1.0 + 1.0e3 * 1.0e-10));
    if (dbdr > 1) {
      const double dr = (Rn - Rx) / (1.0 * dbdr);
      for (int ii = 1; ii <= dbdr - 1; ii++) ring(Rx + ii * dr);
    }
  }
  auto& r = cam.rays_r;
  auto& ri = cam.ri;
  const int nrr = cam.nrr;
  for (int ir = 1; ir <= nrr; ir++) ri[ir] = 0.5 * (r[ir] + r[ir - 1]);
  ri[nrr + 1] = m.R[m.nr + 1];
  for (int ir = 1; ir <= nrr - 1; ir++)
    if (r[ir] - ri[ir] > 2 * (ri[ir + 1] - r[ir])) ri[ir] = r[ir] - 2 * (ri[ir + 1] - r[ir]);
  if (ri[1] < rstar) {
    if (r[1] < rstar) { err = "camera: internal error in the ring layout"; return -1; }
    ri[1] = rstar;
  }
  return 0;
}

int setup_pv_camera(const Model& m, const PVSpec& spec, double incl, PVCamera& cam, std::string& err) {
  const int nx = spec.nx, ny = spec.ny;
  if (nx < 2 || ny < 2 || nx % 2 || ny % 2) { err = "position-velocity image: nx and ny must be even and positive"; return -1; }
  if ((long long)nx * ny > 64LL * 1024 * 1024) { err = "position-velocity image: more than 2^26 pixels"; return -1; }
  // pixel size: the file gives the full image size, halved and divided by half the pixel
  // count (telescope.F:197-200)
  const double hx = spec.szimx * 0.5, hy = spec.szimy * 0.5;
  cam.spx = hx / (nx * 0.5);
  cam.spy = hy / (ny * 0.5);
  if (!(cam.spx > 0.0) || !(cam.spy > 0.0)) { err = "position-velocity image: pixel size must be positive"; return -1; }
  if (spec.addstar > 0 && (spec.xoff != 0.0 || spec.yoff != 0.0)) {
    err = "position-velocity image: the unresolved star can only be added to a star-centred image (offsets 0)";
    return -1;
  }
  if (incl < 1.0e-1) incl = (double)0.1f;   // (telescope.F:2289-2300, no absolute value here)
  cam.incl_rad = incl;
  cam.theta0 = incl + 1.0e-4;
  cam.nx = nx; cam.ny = ny;
  const double sinth0 = std::sin(cam.theta0);
  const int nxh = nx / 2, nyh = ny / 2;
  const int npix = nx * ny;
  cam.nrays = npix + (spec.addstar > 0 ? 1 : 0);
  cam.x0.assign(cam.nrays, 0.0);
  cam.z0.assign(cam.nrays, 0.0);
  cam.b.assign(npix, 0.0);
  int ir = 0;
  for (int ix = 1; ix <= nx; ix++) {
    for (int iy = 1; iy <= ny; iy++) {
      double xc = (ix - nxh - 0.5) * cam.spx - spec.xoff;
      const double yc = (iy - nyh - 0.5) * cam.spy - spec.yoff;
      const double rc = std::sqrt(xc * xc + yc * yc);
      if (xc == 0.0) xc = xc + 0.001 * cam.spx;
      double pc = std::atan(yc / xc) - spec.phioff;
      if (xc < 0.0) pc = pc + 3.14159265359;
      while (pc < 0.0) pc = pc + 6.28318530718;
      while (pc >= 6.28318530718) pc = pc - 6.28318530718;
      const double zh = -std::sin(pc) / sinth0;
      double dum = 1.0 - zh * zh * sinth0 * sinth0;
      dum = dum + 1.0e-4;
      if (dum < 0.0) { err = "position-velocity image: negative discriminant in the ray setup"; return -1; }
      const double xh = std::cos(pc) > 0.0 ? std::sqrt(dum) : -std::sqrt(dum);
      cam.x0[ir] = rc * xh;
      cam.z0[ir] = rc * zh;
      cam.b[ir] = rc;
      ir++;
    }
  }
  // central ray (x0 = z0 = 0) for the unresolved star, used when the pixels are larger
  // than the star (telescope.F:2404-2441)
  cam.starunres = spec.addstar > 0 && cam.spx * cam.spx + cam.spy * cam.spy > m.rstar * m.rstar;
  cam.srat = (3.14159265 * (m.rstar * m.rstar)) / (4.0 * cam.spx * cam.spy);
  cam.rmax = m.R[m.nr + 1];
  return 0;
}

int prepare_line(const Model& m, int iline, bool scaled, LinePrep& lp, std::string& err, bool with_isrf) {
  if (iline < 1 || iline > (int)m.lfreq.size()) { err = "line index out of range"; return -1; }
  const int il = iline - 1, ncell = m.ncell(), nfr = m.nfr;
  lp.lfreq = m.lfreq[il];
  lp.nu0 = std::fabs(lp.lfreq);
  lp.Bud = 6.78171833781e46 * m.Aud[il] / (lp.lfreq * lp.lfreq * lp.lfreq);
  lp.Bdu = lp.Bud * (m.gdeg[m.lup[il] - 1] / m.gdeg[m.ldn[il] - 1]);
  const double molpg = 1.0 / (m.umass * 1.6726e-24);
  // passband (line.F:427-545)
  const double passb = 3.33567e-6 * lp.nu0 * m.vmax, nu1 = 0.0 - passb, dnu = 2.0 * passb / (nfr - 1.0);
  lp.dnu.resize(nfr); lp.velo.resize(nfr); lp.wch.resize(nfr); lp.star.resize(nfr);
  for (int k = 0; k < nfr; k++) {
    lp.dnu[k] = nu1 + k * dnu;
    lp.velo[k] = lp.dnu[k] / lp.lfreq;
    lp.wch[k] = lp.dnu[k] / (3.33567e-6 * lp.nu0);
    const double fq = lp.nu0 + lp.dnu[k];
    const int i = bracket(m.cnu, fq);
    if (i == 0 || i == m.ncont) lp.star[k] = 0.0;
    else {
      const double wgt = (fq - m.cnu[i - 1]) / (m.cnu[i] - m.cnu[i - 1]);
      lp.star[k] = (1.0 - wgt) * m.starcont[i - 1] + wgt * m.starcont[i];
    }
  }
  // outer boundary type 3: the interstellar field at each channel frequency
  // (line_init_passband_outerbc, line.F:3855-3903). Unlike the stellar table it zeroes the
  // channel whose bracket index equals the channel count (freq_nr), not the frequency count;
  // above the last frequency (other than that) the reference reads past its table.
  lp.isrf.clear();
  if (m.outer_bc == 3 && with_isrf) {
    lp.isrf.resize(nfr);
    for (int k = 0; k < nfr; k++) {
      const double fq = lp.nu0 + lp.dnu[k];
      const int i = bracket(m.cnu, fq);
      if (i == 0 || i == nfr) lp.isrf[k] = 0.0;
      else if (i >= m.ncont) {
        err = "line " + std::to_string(iline) + ": channel " + std::to_string(k + 1) +
              " lies above the last frequency of frequency.inp, where the reference's outer boundary "
              "type 3 interpolates past the end of interstellfield.inp";
        return -1;
      } else {
        const double wgt = (fq - m.cnu[i - 1]) / (m.cnu[i] - m.cnu[i - 1]);
        lp.isrf[k] = (1.0 - wgt) * m.isrf[i - 1] + wgt * m.isrf[i];
      }
    }
  }
  // grey dust at the line centre (line.F:3502-3677)
  std::vector<double> jd(ncell, 0.0), ad(ncell, 0.0);
  if (m.line_dust) {
    const int i = bracket(m.cnu, lp.lfreq);
    if (i != 0 && i != m.ncont) {
      const double wgt = (lp.lfreq - m.cnu[i - 1]) / (m.cnu[i] - m.cnu[i - 1]);
      for (int c = 0; c < ncell; c++) {
        double src = 0.0, alp = 0.0;
        for (int s = 0; s < m.nspec; s++)
          for (int z = 0; z < m.nsize[s]; z++) {
            const double* ka = &m.kabs[((size_t)s * 4 + z) * m.ncont];
            const double kw = wgt * ka[i] + (1.0 - wgt) * ka[i - 1];
            const double dr = m.drho[(size_t)s * ncell + c];
            src = src + dr * kw * bplanck(m.dtemp[((size_t)s * 4 + z) * ncell + c], lp.lfreq);
            alp = alp + dr * kw;
          }
        if (!m.scat.empty())
          src = src + wgt * m.scat[(size_t)i * ncell + c] + (1.0 - wgt) * m.scat[(size_t)(i - 1) * ncell + c];
        for (int s = 0; s < m.nspec; s++)
          for (int z = 0; z < m.nsize[s]; z++) {
            const double* ks = &m.ksca[((size_t)s * 4 + z) * m.ncont];
            const double kw = wgt * ks[i] + (1.0 - wgt) * ks[i - 1];
            alp = alp + m.drho[(size_t)s * ncell + c] * kw;
          }
        jd[c] = src; ad[c] = alp;
      }
    }
  }
  // emissivity / extinction factors per cell: j = jf * phi, alpha = af * phi
  const double C1 = 5.27296241956e-28 * lp.lfreq * m.Aud[il];
  const double C2 = 5.27296241956e-28 * lp.lfreq;
  std::vector<double> jf(ncell), af(ncell);
  lp.nsum.resize(ncell);
  const int lu = m.lup[il] - 1, ld = m.ldn[il] - 1;
  for (int c = 0; c < ncell; c++) {
    const double nup = m.pop[(size_t)c * m.nlev + lu] * m.abun[c] * m.rho[c] * molpg;
    const double ndn = m.pop[(size_t)c * m.nlev + ld] * m.abun[c] * m.rho[c] * molpg;
    jf[c] = C1 * nup;
    af[c] = C2 * (ndn * lp.Bdu - nup * lp.Bud);
    lp.nsum[c] = nup + ndn;
    if (af[c] < 0.0) lp.mase = true;
  }
  // start intensity at the outer boundary (telescope.F:3989-4028)
  double istart = 0.0;
  if (m.outer_bc == 2) {
    const double fq = lp.lfreq, temp = 2.728;
    istart = 1.47455253991e-47 * (fq * fq * fq) / (std::exp(4.7991598e-11 * fq / temp) - 1.0);
  }
  // intensity scale keeping the FP32 walk away from the bottom of its exponent range:
  // the largest source function of the grid (dust or line, profile-independent)
  double scale = 1.0;
  if (scaled) {
    double smax = 0.0;
    for (int c = 0; c < ncell; c++) {
      if (ad[c] > 0.0) smax = std::max(smax, jd[c] / ad[c]);
      if (af[c] > 0.0) smax = std::max(smax, jf[c] / af[c]);
    }
    for (double v : lp.star) smax = std::max(smax, v);
    for (double v : lp.isrf) smax = std::max(smax, v);
    smax = std::max(smax, istart);
    if (smax > 0.0 && std::isfinite(smax)) scale = smax;
  }
  lp.scale = scale;
  lp.istart = istart / scale;
  for (auto& v : lp.star) v /= scale;
  for (auto& v : lp.isrf) v /= scale;
  lp.tab.resize((size_t)ncell * 4);
  for (int c = 0; c < ncell; c++) {
    lp.tab[4 * (size_t)c + 0] = jf[c] / scale;
    lp.tab[4 * (size_t)c + 1] = af[c];
    lp.tab[4 * (size_t)c + 2] = jd[c] / scale;
    lp.tab[4 * (size_t)c + 3] = ad[c];
  }
  lp.cphi = 0.56419583546 / (3.33567e-6 * lp.nu0);
  return 0;
}

// gfortran Ew.d output: 0.ddddE+ee, the leading zero dropped when it does not fit
static std::string fmt_e(double v, int w, int d) {
  const bool neg = std::signbit(v) && v != 0.0 ? true : (v < 0);
  const double a = std::fabs(v);
  std::string dig;
  int ex = 0;
  if (a == 0.0) dig.assign(d, '0');
  else {
    char tmp[64];
    std::snprintf(tmp, sizeof tmp, "%.*e", d - 1, a);
    for (const char* p = tmp; *p && *p != 'e'; p++) if (*p >= '0' && *p <= '9') dig.push_back(*p);
    ex = std::atoi(std::strchr(tmp, 'e') + 1) + 1;
  }
  char expo[16];
  if (std::abs(ex) <= 99) std::snprintf(expo, sizeof expo, "E%c%02d", ex < 0 ? '-' : '+', std::abs(ex));
  else std::snprintf(expo, sizeof expo, "%c%03d", ex < 0 ? '-' : '+', std::abs(ex));
  const bool lead0 = d + 6 + (neg ? 1 : 0) <= w;
  std::string body = std::string(neg ? "-" : "") + (lead0 ? "0" : "") + "." + dig + expo;
  if ((int)body.size() > w) return std::string(w, '*');
  return std::string(w - body.size(), ' ') + body;
}

// gfortran ESw.d output: d.dddE+ee (the E dropped for three-digit exponents)
static std::string fmt_es(double v, int w, int d) {
  const bool neg = v < 0 || (v == 0.0 && std::signbit(v));
  const double a = std::fabs(v);
  char tmp[64];
  std::snprintf(tmp, sizeof tmp, "%.*e", d, a);
  std::string mant(tmp, std::strchr(tmp, 'e'));
  int ex = std::atoi(std::strchr(tmp, 'e') + 1);
  if (a == 0.0) ex = 0;
  char expo[16];
  if (std::abs(ex) <= 99) std::snprintf(expo, sizeof expo, "E%c%02d", ex < 0 ? '-' : '+', std::abs(ex));
  else std::snprintf(expo, sizeof expo, "%c%03d", ex < 0 ? '-' : '+', std::abs(ex));
  std::string body = std::string(neg ? "-" : "") + mant + expo;
  if ((int)body.size() > w) return std::string(w, '*');
  return std::string(w - body.size(), ' ') + body;
}

// gfortran list-directed output of a default integer: a blank and I11
static std::string fmt_list_int(int v) {
  char b[32];
  std::snprintf(b, sizeof b, " %11d", v);
  return b;
}

// gfortran list-directed output of a REAL(8): a blank, then G25.17E3 with scale factor 1P
// in E form (F form with 17 significant digits and 5 trailing blanks for 0.1 <= |v| < 1e17)
static std::string fmt_list_real(double v) {
  const bool neg = std::signbit(v);
  const double a = std::fabs(v);
  char tmp[64];
  std::snprintf(tmp, sizeof tmp, "%.16e", a);
  const int ex = std::atoi(std::strchr(tmp, 'e') + 1);   // exponent of the 17-digit rounding
  std::string body;
  bool fform = a == 0.0 || (ex >= -1 && ex <= 16);
  if (fform) {
    const int k = a == 0.0 ? 1 : ex + 1;                  // digits before the point
    char f[64];
    std::snprintf(f, sizeof f, "%.*f", 17 - k, a);
    body = std::string(neg ? "-" : "") + f + (k == 17 ? "." : "");
    body = std::string(body.size() < 20 ? 20 - body.size() : 0, ' ') + body + "     ";
  } else {
    std::string mant(tmp, std::strchr(tmp, 'e'));
    char e[16];
    std::snprintf(e, sizeof e, "E%c%03d", ex < 0 ? '-' : '+', std::abs(ex));
    body = std::string(neg ? "-" : "") + mant + e;
    body = std::string(body.size() < 25 ? 25 - body.size() : 0, ' ') + body;
  }
  return " " + body;
}

std::string imcir_file_name(const Model& m, int iline) {
  if (iline < 1 || iline > 99) return std::string();
  return "lineposvelcirc_" + m.molname + "_" + std::to_string(iline) + ".dat";
}

int write_imcir_file(const std::string& path, const Model& m, const Camera& cam, int iline, const double* img,
                     const unsigned char* mask, std::string& err) {
  FILE* fp = std::fopen(path.c_str(), "w");
  if (!fp) { err = "cannot write " + path; return -1; }
  const int il = iline - 1, nfr = m.nfr, nphi = cam.nphi, nrr = cam.nrr;
  const double nu0 = std::fabs(m.lfreq[il]);
  const double passb = 3.33567e-6 * nu0 * m.vmax, dnu = 2.0 * passb / (nfr - 1.0);
  std::fprintf(fp, "%s\n", fmt_list_int(nfr).c_str());   // telescope.F:1614
  for (int k = 0; k < nfr; k++) {                          // telescope.F:1346-1373
    if (k == 0) {
      std::fprintf(fp, "%s\n%s%s\n", fmt_list_real(nu0).c_str(), fmt_list_int(nphi).c_str(), fmt_list_int(nrr).c_str());
      for (int ir = 1; ir <= nrr + 1; ir++) std::fprintf(fp, "%s\n", fmt_e(cam.ri[ir], 12, 6).c_str());
      for (int ir = 1; ir <= nrr + 1; ir++) std::fprintf(fp, "%s\n", fmt_e(ir <= nrr ? cam.rays_r[ir] : 0.0, 12, 6).c_str());
    }
    const double velo = (-passb + k * dnu) / nu0;
    std::fprintf(fp, "        \n%s\n        \n%s\n        \n", fmt_list_real(velo * 2.99792458e5).c_str(),
                 fmt_list_real(img[k]).c_str());
    for (int ip = 0; ip < nphi; ip++)
      for (int ir = 1; ir <= nrr; ir++) {
        const size_t o = (size_t)(1 + (ir - 1) * nphi + ip) * nfr + k;
        std::fprintf(fp, "%s  %1d\n", fmt_e(img[o], 10, 4).c_str(), (int)mask[o]);
      }
  }
  std::fclose(fp);
  return 0;
}

std::string posvel_file_name(const Model& m, int iline) {
  if (iline < 1 || iline > 99) return std::string();
  return "lineposvel_" + m.molname + "_" + std::to_string(iline) + ".dat";
}

int write_posvel_file(const std::string& path, const Model& m, const PVCamera& cam, const PVSpec& spec, int iline,
                      const double* I, const double* tau, std::string& err) {
  FILE* fp = std::fopen(path.c_str(), "w");
  if (!fp) { err = "cannot write " + path; return -1; }
  const int il = iline - 1;
  const double lf = m.lfreq[il], nu0 = std::fabs(lf);
  const double passb = 3.33567e-6 * nu0 * m.vmax, dnu = 2.0 * passb / (m.nfr - 1.0);
  // header (telescope.F:1965-1984); the distance is 1 pc (main.F:206)
  std::fprintf(fp, "\n%2d\n%-80s\n%-80s\n", 1, m.molname.c_str(), ("./" + m.molfile).c_str());
  std::fprintf(fp, "%s%s%7.3f\n", fmt_es(1.0, 12, 4).c_str(), fmt_es(m.radvelo, 12, 4).c_str(),
               m.incl_rad * 57.2957795132);
  std::fprintf(fp, "%5d%5d\n%s\n%5d\n", m.lup[il], m.ldn[il], fmt_es(lf, 12, 4).c_str(), m.nfr);
  std::fprintf(fp, "%5d%5d%s%s%7.3f%s%s\n  \n", cam.nx, cam.ny, fmt_es(cam.spx, 12, 4).c_str(),
               fmt_es(cam.spy, 12, 4).c_str(), spec.phioff, fmt_es(spec.xoff, 12, 4).c_str(),
               fmt_es(spec.yoff, 12, 4).c_str());
  for (int k = 0; k < m.nfr; k++) {   // velocities (telescope.F:1989-1995)
    const double fq = nu0 + (-passb + k * dnu);
    const double velo = -2.99792458e5 * (fq - lf) / lf + m.radvelo;
    std::fprintf(fp, "%s \n", fmt_e(velo, 10, 3).c_str());
  }
  std::fprintf(fp, "  \n");
  // per channel, iy outer and ix inner: brightness temperature-like 3.25465503368e36 I / nu0^2
  // and the line-of-sight optical depth (telescope.F:2006-2016)
  const size_t npix = (size_t)cam.nx * cam.ny;
  for (int k = 0; k < m.nfr; k++) {
    const double* Ik = I + (size_t)k * npix;
    const double* tk = tau + (size_t)k * npix;
    for (size_t p = 0; p < npix; p++) {
      const double temp = (3.25465503368e36 / (lf * lf)) * Ik[p];
      std::fprintf(fp, "%s %s \n", fmt_es(temp, 12, 5).c_str(), fmt_es(tk[p], 12, 5).c_str());
    }
    std::fprintf(fp, "  \n");
  }
  std::fclose(fp);
  return 0;
}

int write_spectrum_file(const std::string& path, const Model& m, const Camera& cam, const std::vector<int>& lines,
                        const std::vector<double>& flux, std::string& err) {
  FILE* fp = std::fopen(path.c_str(), "w");
  if (!fp) { err = "cannot write " + path; return -1; }
  std::fprintf(fp, "%2d\n%2d\n%-80s\n%-80s\n%10d\n%10d\n", 1, m.style, m.molname.c_str(),
               ("./" + m.molfile).c_str(), (int)lines.size(), m.nfr);
  std::fprintf(fp, "%s%s%7.3f\n", fmt_e(1.0, 12, 4).c_str(), fmt_e(m.radvelo, 12, 4).c_str(),
               cam.incl_rad * 57.2957795132);
  for (size_t li = 0; li < lines.size(); li++) {
    const int il = lines[li] - 1;
    const double lf = m.lfreq[il], nu0 = std::fabs(lf);
    const double passb = 3.33567e-6 * nu0 * m.vmax, dnu = 2.0 * passb / (m.nfr - 1.0);
    std::fprintf(fp, "\n%5d%5d\n%s\n%s\n%5d\n  \n", m.lup[il], m.ldn[il], fmt_e(lf, 14, 9).c_str(),
                 fmt_e(0.0, 10, 5).c_str(), m.nfr);
    for (int k = m.nfr - 1; k >= 0; k--) {
      const double fq = nu0 + (-passb + k * dnu);
      const double velo = -2.99792458e5 * (fq - lf) / lf + m.radvelo;
      std::fprintf(fp, "%s %s\n", fmt_e(velo, 13, 6).c_str(), fmt_e(flux[li * m.nfr + k], 13, 6).c_str());
    }
  }
  std::fclose(fp);
  return 0;
}

}  // namespace rl
