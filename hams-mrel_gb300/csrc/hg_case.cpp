// A whole HAMS run from its input deck: the reader of ControlFile.in and the
// panel meshes (ReadControlFile, src/InputFiles.f90:46-224; ReadBodyMesh /
// ReadWTPLMesh and their multi-body forms, src/ReadPanelMesh.f90 and
// src/ReadPanelMeshMulti.f90; the generalized-mode files of CalNormals,
// src/ReadPanelMesh.f90:150-183), the frequency loop of HAMS_Prog
// (src/HAMS_Prog.f90:255-304 single body, :613-733 multi-body) on the
// device through hg_solve_sweep / hg_solve_frequency, and the writers of the
// HAMS-format and WAMIT-format result files (RFORCE / EFORCE,
// src/PotentWavForce.f90:100-218, src/PotentWavForceMulti.f90:100-223; the pressure and
// elevation files of OutputPressureElevation_Radiation / _Diffraction,
// src/PressureElevation.f90:336-470, and of their multi-body forms with the
// incident-wave file, src/PressureElevationMulti.f90:407-587), and the motion equations
// of SolveMotion / SolveMotionMulti (src/SolveMotion.f90, src/SolveMotionMulti.f90)
// with the hydrostatic decks of ReadHydroStatic(Multi) (src/HydroStatic.f90,
// src/HydroStaticMulti.f90): Motion.4 and Hydrostat.hst; and the single-body
// Hydrostar-format files (src/PrintOutput.f90).  Host code: parsing,
// orchestration, the 6 NBODY x 6 NBODY motion solves per frequency and
// heading, and formatting; every boundary-integral solve runs on the GPU.
//
// The writers reproduce the reference's Fortran edit descriptors (Fw.d,
// Ew.d, ESw.d, Iw) character for character, including its choices that a
// reader might not expect: the WAMIT phase column of ExcForce.3 is
// ATAN2D(...) * 180 / PI (degrees converted once more), zero- and infinite-
// frequency entries write added mass only, and single-body radiation pressure
// lines are written only for field points below the free surface (the
// multi-body radiation records hold elevations for points on it).
#include <sys/stat.h>
#include <sys/types.h>

#include <algorithm>
#include <array>
#include <cctype>
#include <cmath>
#include <complex>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "hamsgpu.h"

namespace {

constexpr double kPi = 3.141592653589793;
constexpr int kNk = 200;  // dispersion roots per finite-depth frequency

struct CaseError {
  int code;
  std::string msg;
};

[[noreturn]] void raise(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  throw CaseError{code, buf};
}

std::vector<std::string> read_lines(const std::string& path, bool required = true) {
  std::ifstream f(path);
  if (!f) {
    if (required) raise(-2, "cannot open %s", path.c_str());
    return {};
  }
  std::vector<std::string> out;
  std::string s;
  while (std::getline(f, s)) {
    if (!s.empty() && s.back() == '\r') s.pop_back();
    out.push_back(s);
  }
  return out;
}

bool file_exists(const std::string& p) {
  struct stat st;
  return stat(p.c_str(), &st) == 0 && S_ISREG(st.st_mode);
}

// Fortran formatted input of one field: blanks are ignored (BLANK='NULL'),
// an all-blank field reads as zero, D exponents are accepted and a real
// without a decimal point or exponent carries `implied` decimals (Fw.d).
std::string field(const std::string& line, size_t skip, size_t width) {
  if (line.size() <= skip) return std::string();
  return line.substr(skip, width);
}

std::string squeeze(const std::string& s) {
  std::string t;
  for (char c : s)
    if (c != ' ' && c != '\t') t += (c == 'D' || c == 'd') ? 'E' : c;
  return t;
}

double f_real(const std::string& s, int implied) {
  const std::string t = squeeze(s);
  if (t.empty()) return 0.0;
  char* end = nullptr;
  if (t.find_first_of(".eE") != std::string::npos) {
    const double v = std::strtod(t.c_str(), &end);
    if (end == t.c_str()) raise(-3, "not a number: '%s'", s.c_str());
    return v;
  }
  const long long i = std::strtoll(t.c_str(), &end, 10);
  if (end == t.c_str()) raise(-3, "not a number: '%s'", s.c_str());
  return (double)i / std::pow(10.0, implied);
}

int f_int(const std::string& s) {
  const std::string t = squeeze(s);
  if (t.empty()) return 0;
  char* end = nullptr;
  const long v = std::strtol(t.c_str(), &end, 10);
  if (end == t.c_str() || *end) raise(-3, "not an integer: '%s'", s.c_str());
  return (int)v;
}

// List-directed values (whitespace or comma separated, D exponents).
std::vector<std::string> tokens(const std::string& line) {
  std::vector<std::string> out;
  std::string cur;
  for (char c : line) {
    if (c == ' ' || c == '\t' || c == ',') {
      if (!cur.empty()) out.push_back(cur), cur.clear();
    } else {
      cur += c;
    }
  }
  if (!cur.empty()) out.push_back(cur);
  return out;
}

double l_real(const std::string& tok) {
  std::string t = tok;
  for (char& c : t)
    if (c == 'D' || c == 'd') c = 'E';
  char* end = nullptr;
  const double v = std::strtod(t.c_str(), &end);
  if (end == t.c_str()) raise(-3, "not a number: '%s'", tok.c_str());
  return v;
}

struct Cursor {
  const std::vector<std::string>& lines;
  size_t i = 0;
  explicit Cursor(const std::vector<std::string>& l) : lines(l) {}
  const std::string& next() {
    if (i >= lines.size()) raise(-3, "ControlFile.in ends early (line %zu)", i + 1);
    return lines[i++];
  }
  // READ(1,*) of n reals: as many records as needed
  std::vector<double> list(int n) {
    std::vector<double> v;
    while ((int)v.size() < n) {
      for (const auto& t : tokens(next())) {
        if ((int)v.size() < n) v.push_back(l_real(t));
      }
    }
    return v;
  }
};

}  // namespace

struct hg_case {
  std::string dir;
  // control (ReadControlFile)
  double h = 0;
  int sybo = 0, inft = 0, ouft = 0, nper = 0, nbody = 1, isol = 1, irsp = 0, nthread = 0, isolv = 1;
  double refl = 1;
  std::vector<double> wvnb;                  // frequency-list entries (the first two unused when sybo = 1)
  std::vector<std::array<double, 4>> lcs;    // multi-body local frames (x, y, z, angle)
  std::vector<double> headings;              // degrees
  std::vector<std::array<double, 3>> xr;     // rotation centres
  std::vector<double> xfp;                   // field points, 3 per point
  bool sep = false;                          // separate_wamit_diffraction_radiation_files (several bodies)
  // combined mesh (BuildCombinedArrays order: body after body)
  int n = 0, nl = 0, ntnd = 0;
  std::vector<double> nodes, xyz_p, ds, pnsz, dxyz, lid;  // column-major (ntnd x 3, n x 3, n, n, n x 6, nl x 3)
  std::vector<int> ncon, ncn, ranges;                     // n x 4 column-major (1-based), n, 2 x nbody (1-based)
  // per frequency (CalWaveProperts)
  std::vector<double> v, wk, w1, tp, wl, oufr, wvn;       // wvn: nper x kNk (finite depth)
  // hydrostatic decks (per body, 6 x 6 row-major each): mass, external linear and
  // quadratic damping, hydrostatic and external restoring
  bool hydro = false;
  std::vector<double> matx, blnr, bqdr, crs, kstf;
  std::string err;
};

namespace {

void read_control(hg_case* c) {
  const auto lines = read_lines(c->dir + "/ControlFile.in");
  Cursor in(lines);
  in.next();
  in.next();
  c->h = f_real(field(in.next(), 14, 30), 15);
  in.next();
  in.next();
  c->sybo = f_int(field(in.next(), 27, 16));
  c->inft = f_int(field(in.next(), 25, 16));
  c->ouft = f_int(field(in.next(), 25, 17));
  int npet = f_int(field(in.next(), 26, 16));
  if (c->inft < 1 || c->inft > 5) raise(-3, "Input_frequency_type %d (1..5 expected)", c->inft);
  if (c->ouft < 1 || c->ouft > 5) raise(-3, "Output_frequency_type %d (1..5 expected)", c->ouft);
  const int ifs = (c->sybo == 1) ? 2 : 0;
  c->wvnb.assign(ifs, 0.0);
  if (npet > 0) {
    const auto vals = in.list(npet);
    c->wvnb.insert(c->wvnb.end(), vals.begin(), vals.end());
  } else if (npet < 0) {
    npet = -npet;
    const double wk1 = f_real(field(in.next(), 27, 30), 15);
    const double dwk = f_real(field(in.next(), 19, 30), 15);
    for (int i = ifs + 1; i <= ifs + npet; ++i) c->wvnb.push_back(wk1 + (i - ifs - 1) * dwk);
  }
  c->nper = (int)c->wvnb.size();
  in.next();
  in.next();
  const std::string body_check = in.next();
  c->nbody = (body_check.find("multi") != std::string::npos) ? f_int(field(in.next(), 24, 16)) : 1;
  if (c->nbody < 1) raise(-3, "Number_of_bodies %d", c->nbody);
  if (c->nbody > 1) {
    for (int b = 0; b < c->nbody; ++b) {
      const std::string& ln = in.next();
      std::array<double, 4> l;
      for (int k = 0; k < 4; ++k) l[k] = f_real(field(ln, 26 + 12 * k, 12), 3);
      c->lcs.push_back(l);
    }
    in.next();
    in.next();
    in.next();
  }
  int nbeta = f_int(field(in.next(), 23, 16));
  if (nbeta > 0) {
    c->headings = in.list(nbeta);
  } else if (nbeta < 0) {
    nbeta = -nbeta;
    const double b1 = f_real(field(in.next(), 20, 30), 15);
    const double db = f_real(field(in.next(), 17, 30), 15);
    for (int i = 0; i < nbeta; ++i) c->headings.push_back(b1 + i * db);
  }
  in.next();
  in.next();
  for (int b = 0; b < c->nbody; ++b) {
    const std::string& ln = in.next();
    std::array<double, 3> x;
    for (int k = 0; k < 3; ++k) x[k] = f_real(field(ln, 28 + 12 * k, 12), 3);
    c->xr.push_back(x);
  }
  c->refl = f_real(field(in.next(), 26, 30), 15);
  c->isol = f_int(field(in.next(), 26, 16));
  c->irsp = f_int(field(in.next(), 23, 16));
  c->nthread = f_int(field(in.next(), 23, 16));
  if (c->isol != 1 && c->isol != 2) raise(-3, "Wave_diffrac_solution %d (1 or 2 expected)", c->isol);
  if (c->irsp != 0 && c->irsp != 1) raise(-3, "If_remove_irr_freq %d (0 or 1 expected)", c->irsp);
  // optional Solver_type line, then the field points
  if (in.i < lines.size() && lines[in.i].find("Solver_type") != std::string::npos) {
    const std::string& ln = in.next();
    try {
      c->isolv = f_int(field(ln, 26, 16));
    } catch (const CaseError&) {
      c->isolv = 1;
    }
    if (c->isolv < 1 || c->isolv > 2) c->isolv = 1;
  }
  if (in.i + 2 < lines.size()) {
    in.next();
    in.next();
    const int nfp = f_int(field(in.next(), 27, 16));
    for (int p = 0; p < nfp; ++p) {
      const auto v = in.list(3);
      c->xfp.insert(c->xfp.end(), v.begin(), v.end());
    }
    // WAMIT output layout (InputFiles.f90:204-220): two lines on, an optional
    // "separate..." line with the flag at column 51 (read with an I edit
    // descriptor into a LOGICAL: odd is true); one body never separates
    if (in.i + 3 <= lines.size()) {
      in.next();
      in.next();
      const std::string& ln = in.next();
      if (ln.find("separate") != std::string::npos || ln.find("Separate") != std::string::npos) {
        try {
          c->sep = (f_int(field(ln, 50, 16)) & 1) != 0;
        } catch (const CaseError&) {
          c->sep = false;
        }
      }
    }
  }
  if (c->nbody == 1) c->sep = false;
}

struct Pnl {
  int nelem = 0, ntnd = 0;
  std::vector<double> nodes;  // ntnd x 3 column-major
  std::vector<int> ncon, ncn; // nelem x 4 column-major (1-based, local)
};

Pnl read_pnl(const std::string& path, const std::array<double, 4>* lcs, bool lid) {
  const auto lines = read_lines(path);
  if (lines.size() < 7) raise(-4, "%s: too short for a panel mesh", path.c_str());
  const auto hd = tokens(lines[3]);
  if (hd.size() < 4) raise(-4, "%s: line 4 must hold NELEM NTND ISX ISY", path.c_str());
  Pnl p;
  p.nelem = f_int(hd[0]);
  p.ntnd = f_int(hd[1]);
  const int isx = f_int(hd[2]), isy = f_int(hd[3]);
  if (isx != 0 || isy != 0) raise(-4, "%s: symmetry planes (ISX/ISY) are not supported", path.c_str());
  if (p.nelem <= 0 || p.ntnd <= 0) raise(-4, "%s: no panels or nodes", path.c_str());
  if (lines.size() < (size_t)(6 + p.ntnd + 3 + p.nelem)) raise(-4, "%s: ends before its panels", path.c_str());
  p.nodes.assign((size_t)p.ntnd * 3, 0.0);
  for (int i = 0; i < p.ntnd; ++i) {
    const auto t = tokens(lines[6 + i]);
    if (t.size() < 4) raise(-4, "%s: node line %d", path.c_str(), i + 1);
    double x = l_real(t[1]), y = l_real(t[2]);
    const double z = l_real(t[3]);
    if (lid && std::fabs(z) > 1.0e-10) raise(-4, "%s: Z coordinate is not zero at node %d", path.c_str(), i + 1);
    if (lcs) {
      const double ca = std::cos((*lcs)[3]), sa = std::sin((*lcs)[3]);
      const double gx = 0.0 + (*lcs)[0] + ca * x - sa * y;
      const double gy = 0.0 + (*lcs)[1] + sa * x + ca * y;
      x = gx;
      y = gy;
    }
    p.nodes[i] = x;
    p.nodes[i + p.ntnd] = y;
    p.nodes[i + 2 * (size_t)p.ntnd] = z;
  }
  p.ncon.assign((size_t)p.nelem * 4, 0);
  p.ncn.assign(p.nelem, 0);
  const size_t e0 = 6 + p.ntnd + 3;
  for (int e = 0; e < p.nelem; ++e) {
    const auto t = tokens(lines[e0 + e]);
    if (t.size() < 2) raise(-4, "%s: panel line %d", path.c_str(), e + 1);
    const int nv = f_int(t[1]);
    if ((nv != 3 && nv != 4) || (int)t.size() < 2 + nv) raise(-4, "%s: panel %d has %d vertices", path.c_str(), e + 1, nv);
    p.ncn[e] = nv;
    for (int k = 0; k < nv; ++k) {
      const int id = f_int(t[2 + k]);
      if (id < 1 || id > p.ntnd) raise(-4, "%s: panel %d vertex %d: node %d out of range", path.c_str(), e + 1, k + 1, id);
      p.ncon[e + (size_t)k * p.nelem] = id;
    }
    if (nv == 3) p.ncon[e + 3 * (size_t)p.nelem] = p.ncon[e];
  }
  return p;
}

void read_meshes(hg_case* c) {
  struct Body {
    Pnl hull;
    std::vector<double> xyz, ds, pnsz, dxyz, lid;
    int nl = 0;
  };
  std::vector<Body> bodies(c->nbody);
  for (int b = 0; b < c->nbody; ++b) {
    Body& B = bodies[b];
    const bool multi = c->nbody > 1;
    const std::string sfx = multi ? "_" + std::to_string(b + 1) : "";
    const std::array<double, 4>* lcs = multi ? &c->lcs[b] : nullptr;
    B.hull = read_pnl(c->dir + "/HullMesh" + sfx + ".pnl", lcs, false);
    const int nb = B.hull.nelem;
    B.xyz.resize((size_t)nb * 3);
    B.ds.resize(nb);
    B.pnsz.resize(nb);
    B.dxyz.resize((size_t)nb * 6);
    int rc = hg_panel_geometry(nb, B.hull.ntnd, B.hull.nodes.data(), B.hull.ncon.data(), B.hull.ncn.data(),
                               c->xr[b].data(), B.xyz.data(), B.ds.data(), B.pnsz.data(), B.dxyz.data());
    if (rc) raise(-4, "panel geometry of body %d failed (%d)", b + 1, rc);
    // generalized modes: gen_mod_<body>_<dof>.txt, "panel value" per line
    for (int dof = 1; dof <= 6; ++dof) {
      const std::string gname = c->dir + "/gen_mod_" + std::to_string(b + 1) + "_" + std::to_string(dof) + ".txt";
      if (!file_exists(gname)) continue;
      const auto gl = read_lines(gname);
      for (int k = 0; k < nb && k < (int)gl.size(); ++k) {
        const auto t = tokens(gl[k]);
        if (t.size() < 2) break;
        int pid;
        double val;
        try {
          pid = f_int(t[0]);
          val = l_real(t[1]);
        } catch (const CaseError&) {
          break;
        }
        if (pid < 1 || pid > nb) raise(-4, "%s: panel %d out of range", gname.c_str(), pid);
        B.dxyz[(pid - 1) + (size_t)(dof - 1) * nb] = val;
      }
    }
    if (c->irsp == 1) {
      const std::string wname = c->dir + "/WaterPlaneMesh" + sfx + ".pnl";
      if (!file_exists(wname)) raise(-4, "IRSP = 1 needs %s", wname.c_str());
      Pnl lp = read_pnl(wname, lcs, true);
      B.nl = lp.nelem;
      B.lid.resize((size_t)lp.nelem * 3);
      std::vector<double> lds(lp.nelem), lsz(lp.nelem), ldx((size_t)lp.nelem * 6);
      rc = hg_panel_geometry(lp.nelem, lp.ntnd, lp.nodes.data(), lp.ncon.data(), lp.ncn.data(), c->xr[b].data(),
                             B.lid.data(), lds.data(), lsz.data(), ldx.data());
      if (rc) raise(-4, "panel geometry of lid %d failed (%d)", b + 1, rc);
    }
  }
  c->n = c->nl = c->ntnd = 0;
  for (const Body& B : bodies) {
    c->n += B.hull.nelem;
    c->nl += B.nl;
    c->ntnd += B.hull.ntnd;
  }
  const int n = c->n, nl = c->nl, nt = c->ntnd;
  c->nodes.assign((size_t)nt * 3, 0.0);
  c->ncon.assign((size_t)n * 4, 0);
  c->ncn.assign(n, 0);
  c->xyz_p.assign((size_t)n * 3, 0.0);
  c->ds.assign(n, 0.0);
  c->pnsz.assign(n, 0.0);
  c->dxyz.assign((size_t)n * 6, 0.0);
  c->lid.assign((size_t)nl * 3, 0.0);
  c->ranges.clear();
  int e0 = 0, nd0 = 0, l0 = 0;
  for (const Body& B : bodies) {
    const int nb = B.hull.nelem, tb = B.hull.ntnd;
    for (int i = 0; i < tb; ++i)
      for (int k = 0; k < 3; ++k) c->nodes[(nd0 + i) + (size_t)k * nt] = B.hull.nodes[i + (size_t)k * tb];
    for (int e = 0; e < nb; ++e) {
      c->ncn[e0 + e] = B.hull.ncn[e];
      for (int k = 0; k < 4; ++k) c->ncon[(e0 + e) + (size_t)k * n] = B.hull.ncon[e + (size_t)k * nb] + nd0;
      for (int k = 0; k < 3; ++k) c->xyz_p[(e0 + e) + (size_t)k * n] = B.xyz[e + (size_t)k * nb];
      for (int k = 0; k < 6; ++k) c->dxyz[(e0 + e) + (size_t)k * n] = B.dxyz[e + (size_t)k * nb];
      c->ds[e0 + e] = B.ds[e];
      c->pnsz[e0 + e] = B.pnsz[e];
    }
    for (int e = 0; e < B.nl; ++e)
      for (int k = 0; k < 3; ++k) c->lid[(l0 + e) + (size_t)k * nl] = B.lid[e + (size_t)k * B.nl];
    c->ranges.push_back(e0 + 1);
    c->ranges.push_back(e0 + nb);
    e0 += nb;
    nd0 += tb;
    l0 += B.nl;
  }
}

// ReadHydroStatic(Multi) (src/HydroStatic.f90:41-82): Hydrostatic.in or
// Hydrostatic_<b>.in per body, five 6 x 6 matrices in FORMAT(6(2x,E12.5))
// after a title line each; the centre of gravity is read past.  Decks without
// them run without motions.
void read_hydrostatics(hg_case* c) {
  const int nb = c->nbody;
  std::vector<double>* mats[5] = {&c->matx, &c->blnr, &c->bqdr, &c->crs, &c->kstf};
  for (auto* m : mats) m->assign((size_t)36 * nb, 0.0);
  for (int b = 0; b < nb; ++b) {
    const std::string path = c->dir + "/Hydrostatic" + (nb > 1 ? "_" + std::to_string(b + 1) : std::string()) + ".in";
    if (!file_exists(path)) return;
    const auto lines = read_lines(path);
    size_t i = 3;  // title, centre of gravity, title
    for (auto* m : mats) {
      for (int r = 0; r < 6; ++r) {
        if (i >= lines.size()) raise(-7, "%s ends early", path.c_str());
        const std::string& ln = lines[i++];
        for (int q = 0; q < 6; ++q) (*m)[(size_t)36 * b + 6 * r + q] = f_real(field(ln, 2 + 14 * q, 12), 5);
      }
      ++i;  // the next title
    }
  }
  c->hydro = true;
}

// CalWaveProperts (src/ImplementSubs.f90:40-151) for every entry; TP keeps
// its previous value where the input type does not set it (type 5), as there.
void wave_properties(hg_case* c) {
  const int np = c->nper;
  const bool fin = c->h > 0.0;
  c->v.assign(np, 0.0);
  c->wk.assign(np, 0.0);
  c->w1.assign(np, 0.0);
  c->tp.assign(np, 0.0);
  c->wl.assign(np, 0.0);
  c->oufr.assign(np, 0.0);
  c->wvn.assign(fin ? (size_t)np * kNk : 1, 0.0);
  double tp = 0.0;
  for (int k = 0; k < np; ++k) {
    double v, wk, w1, wl;
    if (c->sybo == 1 && k < 2) {
      v = wk = w1 = (k == 0) ? 0.0 : -1.0;
      tp = (k == 0) ? -1.0 : 0.0;
      wl = tp;
    } else {
      double* roots = fin ? c->wvn.data() + (size_t)k * kNk : nullptr;
      const int rc = hg_wave_properties(c->inft, c->wvnb[k], c->h, kNk, &v, &wk, &w1, roots);
      if (rc) raise(-5, "wave properties of entry %d (%g) failed (%d)", k + 1, c->wvnb[k], rc);
      wl = (c->inft == 5) ? c->wvnb[k] : 2.0 * kPi / wk;
      if (c->inft == 4) tp = c->wvnb[k];
      else if (c->inft != 5) tp = 2.0 * kPi / w1;
    }
    c->v[k] = v;
    c->wk[k] = wk;
    c->w1[k] = w1;
    c->tp[k] = tp;
    c->wl[k] = wl;
    const double o[5] = {v, wk, w1, tp, wl};
    c->oufr[k] = o[c->ouft - 1];
  }
}

// ---------------------------------------------------------------------------
// Fortran edit descriptors
// ---------------------------------------------------------------------------
std::string fit(std::string s, int w) {
  if ((int)s.size() > w) return std::string(w, '*');
  return std::string(w - s.size(), ' ') + s;
}

// Non-finite values as gfortran writes them.
std::string nonfinite(int w, double x) {
  if (std::isnan(x)) return fit("NaN", w);
  const std::string s = (x < 0 ? "-" : "") + std::string(w >= 9 ? "Infinity" : "Inf");
  return fit(s, w);
}

std::string fF(int w, int d, double x) {  // Fw.d
  if (!std::isfinite(x)) return nonfinite(w, x);
  char b[64];
  snprintf(b, sizeof(b), "%.*f", d, x);
  return fit(b, w);
}

std::string fI(int w, int x) {  // Iw
  return fit(std::to_string(x), w);
}

// Decimal digits and exponent of |x| rounded to nd significant digits:
// |x| = 0.D1D2..Dnd x 10^e10.
void sig_digits(double x, int nd, std::string& digits, int& e10) {
  if (x == 0.0) {
    digits.assign(nd, '0');
    e10 = 0;
    return;
  }
  char b[64];
  snprintf(b, sizeof(b), "%.*e", nd - 1, std::fabs(x));  // d.ddd e+XX
  digits.clear();
  const char* p = b;
  for (; *p && *p != 'e'; ++p)
    if (std::isdigit((unsigned char)*p)) digits += *p;
  e10 = std::atoi(p + 1) + 1;
}

std::string exponent(int e, bool with_letter) {
  char b[16];
  const int a = std::abs(e);
  if (a <= 99) snprintf(b, sizeof(b), "%s%c%02d", with_letter ? "E" : "", e < 0 ? '-' : '+', a);
  else snprintf(b, sizeof(b), "%c%03d", e < 0 ? '-' : '+', a);  // Fortran drops the letter for 3 digits
  return b;
}

std::string fE(int w, int d, double x) {  // Ew.d: 0.ddddddE+XX
  if (!std::isfinite(x)) return nonfinite(w, x);
  std::string dg;
  int e;
  sig_digits(x, d, dg, e);
  if (x == 0.0) e = 0;
  std::string s = (x < 0 ? "-" : "") + std::string("0.") + dg + exponent(e, true);
  return fit(s, w);
}

std::string fES(int w, int d, double x) {  // ESw.d: d.ddddddE+XX
  if (!std::isfinite(x)) return nonfinite(w, x);
  std::string dg;
  int e;
  sig_digits(x, d + 1, dg, e);
  if (x != 0.0) e -= 1;
  std::string s = (x < 0 ? "-" : "") + dg.substr(0, 1) + "." + dg.substr(1) + exponent(e, true);
  return fit(s, w);
}

bool special(double tp) { return std::fabs(tp + 1.0) < 1.e-6 || std::fabs(tp) < 1.e-6; }

void make_dir(const std::string& d) {
  if (mkdir(d.c_str(), 0755) != 0 && errno != EEXIST) raise(-6, "cannot create %s", d.c_str());
}

struct Out {
  FILE* f = nullptr;
  Out(const std::string& p) {
    f = std::fopen(p.c_str(), "w");
    if (!f) raise(-6, "cannot write %s", p.c_str());
  }
  ~Out() {
    if (f) std::fclose(f);
  }
  void line(const std::string& s) { std::fprintf(f, "%s\n", s.c_str()); }
};

void write_motions(const hg_case* c, const std::string& wd, const double* amas, const double* bdmp,
                   const double* exfc, double rho, double g, std::vector<std::complex<double>>* dspl_all);
void write_hydrostar(const hg_case* c, const std::string& out, const double* amas, const double* bdmp,
                     const double* exfc, const std::vector<std::complex<double>>* dspl_all);

// amas/bdmp: nper blocks of nd x nd column-major (row = force DOF, column =
// mode); exfc: nper blocks of (nbeta x nd) COMPLEX*16 column-major.
void write_results(const hg_case* c, const std::string& out, const double* amas, const double* bdmp,
                   const double* exfc, double rho, double g) {
  const int nb = c->nbody, nd = 6 * nb, nbeta = (int)c->headings.size(), np = c->nper;
  const std::string hd = out + "/Hams_format", wd = out + "/Wamit_format";
  make_dir(out);
  make_dir(hd);
  make_dir(wd);
  {  // the pressure/elevation files CreateWamitFiles opens in every run (InputFiles.f90:318-338),
     // empty until field points are written into them
    std::vector<std::string> pe;
    if (nb > 1 && c->sep) {
      pe.push_back("PressureElevationDiffraction.6p");
      for (int b = 0; b < nb; ++b) pe.push_back("PressureElevationRadiation_" + std::to_string(b + 1) + ".6p");
    } else {
      pe.push_back("PressureElevation.6p");
    }
    if (nb > 1) pe.push_back("PressureElevationIncidence.6p");
    for (const auto& name : pe) Out empty(wd + "/" + name);
  }
  const double amp = 1.0;
  auto A = [&](int k, int i, int j) { return amas[(size_t)k * nd * nd + i + (size_t)j * nd]; };
  auto B = [&](int k, int i, int j) { return bdmp[(size_t)k * nd * nd + i + (size_t)j * nd]; };
  auto F = [&](int k, int b, int d) {
    const double* p = exfc + 2 * ((size_t)k * nbeta * nd + b + (size_t)d * nbeta);
    return std::complex<double>(p[0], p[1]);
  };
  // OAMASS / ODAMPING (format 1000: F7.3,1x,F7.3,1x,6E14.5), a line per body pair
  for (int md = 0; md < 6; ++md) {
    Out fa(hd + "/OAMASS" + std::to_string(md + 1) + ".txt");
    Out fb(hd + "/ODAMPING" + std::to_string(md + 1) + ".txt");
    for (int k = 0; k < np; ++k)
      for (int m = 0; m < nb; ++m)
        for (int q = 0; q < nb; ++q) {
          std::string la = fF(7, 3, c->wk[k]) + " " + fF(7, 3, c->w1[k]) + " ";
          std::string lb = la;
          for (int j = 0; j < 6; ++j) {
            la += fE(14, 5, A(k, 6 * m + md, 6 * q + j));
            lb += fE(14, 5, B(k, 6 * m + md, 6 * q + j));
          }
          fa.line(la);
          fb.line(lb);
        }
  }
  // OEXFOR (format 1010: F7.3,1x,F7.3,1x,6E14.6 with Re, Im), a line per heading and body
  for (int md = 0; md < 6; ++md) {
    Out fx(hd + "/OEXFOR" + std::to_string(md + 1) + ".txt");
    for (int k = 0; k < np; ++k)
      for (int ib = 0; ib < nbeta; ++ib)
        for (int m = 0; m < nb; ++m) {
          const std::complex<double> e = F(k, ib, 6 * m + md);
          fx.line(fF(7, 3, c->wk[k]) + " " + fF(7, 3, c->w1[k]) + " " + fE(14, 6, e.real()) + fE(14, 6, e.imag()));
        }
  }
  // AmssDamp.1 (format 1020: ES14.6,2I6,2ES14.6): per frequency and body
  // pair (force body outer, mode body inner) the 36 entries, force DOF outer,
  // as RFORCE / RFORCE_MULTI write them.  (The reference rewrites the
  // multi-body file in row-major order over all DOFs afterwards only when its
  // output directory is the default one, ReorderAmssDamp being handed the
  // fixed path Output/Wamit_format/AmssDamp.1; the files it ships keep the
  // order written here.)
  {
    Out f1(wd + "/AmssDamp.1");
    for (int k = 0; k < np; ++k)
      for (int m = 0; m < nb; ++m)
        for (int q = 0; q < nb; ++q)
          for (int a = 0; a < 6; ++a)
            for (int b = 0; b < 6; ++b) {
              const int i = 6 * m + a, j = 6 * q + b;
              std::string s = fES(14, 6, c->oufr[k]) + fI(6, i + 1) + fI(6, j + 1) + fES(14, 6, A(k, i, j) / rho);
              if (!special(c->tp[k])) s += fES(14, 6, B(k, i, j) / (rho * c->w1[k]));
              f1.line(s);
            }
  }
  // ExcForce.3 (format 1030: 2ES14.6,I6,4ES14.6), regular frequencies only
  {
    Out f3(wd + "/ExcForce.3");
    for (int k = 0; k < np; ++k) {
      if (special(c->tp[k])) continue;
      for (int ib = 0; ib < nbeta; ++ib) {
        const double beta = c->headings[ib] * kPi / 180.0;
        for (int m = 0; m < nb; ++m)
          for (int md = 0; md < 6; ++md) {
            const std::complex<double> e = F(k, ib, 6 * m + md);
            const double rel = e.real() / (rho * g * amp), img = e.imag() / (rho * g * amp);
            const double mod = std::abs(e) / (rho * g * amp);
            const double nrel = -img, nimg = -rel;
            const double phs = std::atan2(nimg, nrel) * (180.0 / kPi) * 180.0 / kPi;
            f3.line(fES(14, 6, c->oufr[k]) + fES(14, 6, beta * 180.0 / kPi) + fI(6, 6 * m + md + 1) +
                    fES(14, 6, mod) + fES(14, 6, phs) + fES(14, 6, nrel) + fES(14, 6, nimg));
          }
      }
    }
  }
  std::vector<std::complex<double>> dspl;
  if (c->hydro) write_motions(c, wd, amas, bdmp, exfc, rho, g, &dspl);
  if (nb == 1) write_hydrostar(c, out, amas, bdmp, exfc, c->hydro ? &dspl : nullptr);
}

// ZGESV of the motion equations (6 NBODY unknowns): LU with partial
// pivoting on |re| + |im| (IZAMAX), one right-hand side.
bool zgesv_small(int n, std::vector<std::complex<double>>& a, std::vector<std::complex<double>>& b) {
  auto at = [&](int i, int j) -> std::complex<double>& { return a[(size_t)i + (size_t)j * n]; };
  auto cabs1 = [](std::complex<double> z) { return std::fabs(z.real()) + std::fabs(z.imag()); };
  for (int k = 0; k < n; ++k) {
    int p = k;
    for (int i = k + 1; i < n; ++i)
      if (cabs1(at(i, k)) > cabs1(at(p, k))) p = i;
    if (cabs1(at(p, k)) == 0.0) return false;
    if (p != k) {
      for (int j = 0; j < n; ++j) std::swap(at(k, j), at(p, j));
      std::swap(b[k], b[p]);
    }
    const std::complex<double> r = 1.0 / at(k, k);
    for (int i = k + 1; i < n; ++i) {
      const std::complex<double> l = at(i, k) * r;
      at(i, k) = l;
      for (int j = k + 1; j < n; ++j) at(i, j) -= l * at(k, j);
      b[i] -= l * b[k];
    }
  }
  for (int k = n - 1; k >= 0; --k) {
    std::complex<double> t = b[k];
    for (int j = k + 1; j < n; ++j) t -= at(k, j) * b[j];
    b[k] = t / at(k, k);
  }
  return true;
}

// SolveMotion / SolveMotionMulti: motions DSPL from
//   [-w^2 (M + A) + i w (B + B_lin [+ B_quad w |DSPL|]) + C + K] DSPL = -Im F - i Re F,
// the quadratic damping by fixed-point iteration until sum |dDSPL|/|DSPL| <= 1e-6
// (single body: every component in the sum, as there; several bodies: zero
// components left out, as there); Motion.4 lines for regular frequencies.
void write_motions(const hg_case* c, const std::string& wd, const double* amas, const double* bdmp,
                   const double* exfc, double rho, double g, std::vector<std::complex<double>>* dspl_all) {
  const int nb = c->nbody, nd = 6 * nb, nbeta = (int)c->headings.size(), np = c->nper;
  auto blk = [&](const std::vector<double>& m, int i, int j) {
    const int bi = i / 6, bj = j / 6;
    return bi == bj ? m[(size_t)36 * bi + 6 * (i % 6) + (j % 6)] : 0.0;
  };
  {
    Out fh(wd + "/Hydrostat.hst");  // FORMAT(2I6,2X,ES14.6)
    for (int i = 0; i < nd; ++i)
      for (int j = 0; j < nd; ++j) fh.line(fI(6, i + 1) + fI(6, j + 1) + "  " + fES(14, 6, blk(c->crs, i, j) / (rho * g)));
  }
  double qnorm = 0.0;
  for (double x : c->bqdr) qnorm = std::max(qnorm, std::fabs(x));
  Out f4(wd + "/Motion.4");
  std::vector<std::complex<double>> left((size_t)nd * nd), rhs(nd), dspl(nd), dspl1(nd);
  dspl_all->assign((size_t)np * std::max(nbeta, 1) * nd, std::complex<double>(0.0, 0.0));
  for (int k = 0; k < np; ++k) {
    const double w1 = c->w1[k];
    const double* A = amas + (size_t)k * nd * nd;
    const double* B = bdmp + (size_t)k * nd * nd;
    for (int ib = 0; ib < nbeta; ++ib) {
      const double* F = exfc + 2 * ((size_t)k * nbeta * nd);
      auto build = [&](bool quad) {
        for (int j = 0; j < nd; ++j)
          for (int i = 0; i < nd; ++i) {
            double damp = B[i + (size_t)j * nd] + blk(c->blnr, i, j);
            if (quad) damp += blk(c->bqdr, i, j) * w1 * std::abs(dspl[j]);
            left[(size_t)i + (size_t)j * nd] =
                std::complex<double>(-w1 * w1 * (blk(c->matx, i, j) + A[i + (size_t)j * nd]) + blk(c->crs, i, j) +
                                         blk(c->kstf, i, j),
                                     w1 * damp);
          }
        for (int i = 0; i < nd; ++i) {
          const double* f = F + 2 * (ib + (size_t)i * nbeta);
          rhs[i] = std::complex<double>(-f[1], -f[0]);
        }
      };
      build(false);
      // a singular system leaves NaN motions in the file (the reference's ZGESV result is not checked either)
      const std::complex<double> nan(std::nan(""), std::nan(""));
      bool ok = zgesv_small(nd, left, rhs);
      dspl = rhs;
      if (!ok) std::fill(dspl.begin(), dspl.end(), nan);
      if (ok && qnorm >= 1.e-6) {
        double rerr = 100.0;
        int guard = 0;
        while (rerr > 1.e-6) {
          if (++guard > 10000) break;  // keeps the last iterate (the reference loops until it settles)
          build(true);
          if (!zgesv_small(nd, left, rhs)) {
            std::fill(dspl.begin(), dspl.end(), nan);
            break;
          }
          dspl1 = rhs;
          rerr = 0.0;
          for (int j = 0; j < nd; ++j) {
            const double dj = std::abs(dspl1[j] - dspl[j]), aj = std::abs(dspl1[j]);
            if (nb == 1 || aj > 0.0) rerr += dj / aj;
          }
          dspl = dspl1;
        }
      }
      std::copy(dspl.begin(), dspl.end(), dspl_all->begin() + ((size_t)k * nbeta + ib) * nd);
      if (special(c->tp[k])) continue;  // Motion.4 holds the regular frequencies only
      const double beta = c->headings[ib] * kPi / 180.0;
      for (int md = 0; md < nd; ++md) {
        const int mexp = (md % 6 < 3) ? 2 : 3;
        const double nfac = 1.0 / std::pow(c->refl, mexp);
        const double nrel = dspl[md].real() / nfac, nimg = dspl[md].imag() / nfac;
        const double magn = std::sqrt(nrel * nrel + nimg * nimg);
        const double phs = std::atan2(nimg, nrel) * (180.0 / kPi);
        f4.line(fES(14, 6, c->oufr[k]) + fES(14, 6, beta * 180.0 / kPi) + fI(6, md + 1) + fES(14, 6, magn) +
                fES(14, 6, phs) + fES(14, 6, nrel) + fES(14, 6, nimg));
      }
    }
  }
}

// Hydrostar-format files of a single body (PrintBody_RealVal / PrintBody_CmplxVal
// / PrintEnd, src/PrintOutput.f90; opened by CreateHydrostarFiles,
// src/InputFiles.f90:339-357; written from src/HAMS_Prog.f90:306-331): per
// entry one line FORMAT(F8.4, NBETA ES14.6, NBETA F12.4) of w and, per
// heading, the real value and 0 (AddedMass_ij, WaveDamping_ij) or the
// modulus and the phase ATAN2D(-Re, -Im) in [0, 360) (Excitation_k,
// Motion_k), then two closing lines.
void write_hydrostar(const hg_case* c, const std::string& out, const double* amas, const double* bdmp,
                     const double* exfc, const std::vector<std::complex<double>>* dspl_all) {
  const int nbeta = (int)c->headings.size(), np = c->nper, nd = 6;
  const std::string hd = out + "/Hydrostar_format";
  make_dir(hd);
  const std::string end1 = "#" + std::string(60, '-'), end2 = "#ENDFILE";
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j)
      for (int which = 0; which < 2; ++which) {
        const double* m = which == 0 ? amas : bdmp;
        Out f(hd + "/" + (which == 0 ? "AddedMass_" : "WaveDamping_") + std::to_string(i + 1) + std::to_string(j + 1) +
              ".rao");
        for (int k = 0; k < np; ++k) {
          const double v = m[(size_t)k * nd * nd + i + (size_t)j * nd];
          std::string s = fF(8, 4, c->w1[k]);
          for (int b = 0; b < nbeta; ++b) s += fES(14, 6, v);
          for (int b = 0; b < nbeta; ++b) s += fF(12, 4, 0.0);
          f.line(s);
        }
        f.line(end1);
        f.line(end2);
      }
  auto cmplx_line = [&](int k, const std::complex<double>* vals, size_t stride) {
    std::string s = fF(8, 4, c->w1[k]);
    for (int b = 0; b < nbeta; ++b) s += fES(14, 6, std::abs(vals[b * stride]));
    for (int b = 0; b < nbeta; ++b) {
      const std::complex<double> z = vals[b * stride];
      double phs = std::atan2(-z.real(), -z.imag()) * (180.0 / kPi);
      if (phs < 0.0) phs += 360.0;
      s += fF(12, 4, phs);
    }
    return s;
  };
  std::vector<std::complex<double>> tmp(nbeta);
  for (int md = 0; md < 6; ++md) {
    Out fx(hd + "/Excitation_" + std::to_string(md + 1) + ".rao");
    for (int k = 0; k < np; ++k) {
      for (int b = 0; b < nbeta; ++b) {
        const double* p = exfc + 2 * ((size_t)k * nbeta * nd + b + (size_t)md * nbeta);
        tmp[b] = std::complex<double>(p[0], p[1]);
      }
      fx.line(cmplx_line(k, tmp.data(), 1));
    }
    fx.line(end1);
    fx.line(end2);
    if (!dspl_all) continue;
    Out fm(hd + "/Motion_" + std::to_string(md + 1) + ".rao");
    for (int k = 0; k < np; ++k) fm.line(cmplx_line(k, dspl_all->data() + (size_t)k * nbeta * nd + md, nd));
    fm.line(end1);
    fm.line(end2);
  }
}

// WamitNondimens (src/PressureElevation.f90:336-385).
std::complex<double> wamit_nondim(std::complex<double> vcp, bool pressure, bool diffraction, int md, double tp,
                                  double w1, double refl, double rho, double g) {
  const double amp = 1.0;
  const double nfac = pressure ? (special(tp) ? rho * amp : rho * g * amp) : amp;
  std::complex<double> r;
  if (diffraction) {
    r = vcp / nfac;
  } else {
    const int mexp = (md <= 3) ? 0 : 1;
    if (special(tp)) r = vcp / nfac * amp / std::pow(refl, mexp + 1);
    else r = vcp / nfac * std::complex<double>(0.0, -w1) * amp / std::pow(refl, mexp);
  }
  if (std::abs(r) < 1.e-15) r = 0.0;
  return diffraction ? std::complex<double>(-r.imag(), -r.real()) : std::complex<double>(r.real(), -r.imag());
}

// Incident-wave potential VINP (PatclVelct.f90:42-76) as CalPotentialIncMulti
// uses it (PressureElevationMulti.f90:277-300): zero unless ISOL = 1, and zero
// at the zero- and infinite-frequency entries; deep water if H < 0 or H > 500.
std::complex<double> incident_potential(const hg_case* c, int k, double x, double y, double z, double beta, double g) {
  if (c->isol != 1 || special(c->tp[k])) return 0.0;
  const double wk = c->wk[k], w1 = c->w1[k], h = c->h;
  const double wkx = wk * (x * std::cos(beta) + y * std::sin(beta));
  const std::complex<double> e(std::cos(wkx), std::sin(wkx));
  if (h < 0.0 || h > 500.0) return -g / w1 * std::exp(wk * z) * e;
  return (-w1 / (wk * std::sinh(wk * h))) * std::cosh(wk * (z + h)) * e;
}

// Several bodies: OutputPressureElevation_RadiationMulti / _DiffractionMulti /
// _IncidenceMulti (PressureElevationMulti.f90:407-587) into the files that
// CreateWamitFiles opens (InputFiles.f90:318-338).  Radiation, per point: all
// six modes of every body; one record per body (the first after the
// frequency and point number, the others indented 24 columns), or, with
// separate files, one PressureElevationRadiation_<body>.6p per body.
// Diffraction, per heading and point: the non-dimensional value (2 reals).
// Incidence (PressureElevationIncidence.6p): modulus, phase in degrees, real
// and imaginary parts of the incident wave's value alone.
void write_pe_multi(const hg_case* c, const char* output_dir, const std::vector<double>& pe, double rho, double g) {
  const int np = c->nper, nb = c->nbody, nd = 6 * nb, nbeta = (int)c->headings.size(), nc = nd + nbeta;
  const int nfp = (int)(c->xfp.size() / 3);
  const std::string wd = std::string(output_dir) + "/Wamit_format";
  std::unique_ptr<Out> fcomb, fdif;
  std::vector<std::unique_ptr<Out>> frad;
  if (c->sep) {
    fdif.reset(new Out(wd + "/PressureElevationDiffraction.6p"));
    for (int b = 0; b < nb; ++b) frad.emplace_back(new Out(wd + "/PressureElevationRadiation_" + std::to_string(b + 1) + ".6p"));
  } else {
    fcomb.reset(new Out(wd + "/PressureElevation.6p"));
  }
  Out finc(wd + "/PressureElevationIncidence.6p");
  Out& dif = c->sep ? *fdif : *fcomb;
  for (int k = 0; k < np; ++k) {
    auto val = [&](int p, int q) {
      const double* v = pe.data() + (((size_t)k * nfp + p) * nc + q) * 2;
      return std::complex<double>(v[0], v[1]);
    };
    for (int p = 0; p < nfp; ++p) {
      const bool below = std::fabs(c->xfp[3 * (size_t)p + 2]) > 1.e-6;
      const std::string head = fES(14, 6, c->oufr[k]) + fI(10, p + 1);
      for (int b = 0; b < nb; ++b) {
        std::string s;
        for (int md = 1; md <= 6; ++md) {
          const auto z = wamit_nondim(val(p, 6 * b + md - 1), below, false, md, c->tp[k], c->w1[k], c->refl, rho, g);
          s += fES(14, 6, z.real()) + fES(14, 6, z.imag());
        }
        if (c->sep) frad[b]->line(head + s);
        else fcomb->line((b == 0 ? head : std::string(24, ' ')) + s);
      }
    }
    for (int ib = 0; ib < nbeta; ++ib) {
      const double beta = c->headings[ib] * kPi / 180.0;
      const std::string hb = fES(14, 6, c->oufr[k]) + fES(14, 6, beta * 180.0 / kPi);
      for (int p = 0; p < nfp; ++p) {
        const bool below = std::fabs(c->xfp[3 * (size_t)p + 2]) > 1.e-6;
        const auto z = wamit_nondim(val(p, nd + ib), below, true, 0, c->tp[k], c->w1[k], c->refl, rho, g);
        dif.line(hb + fI(10, p + 1) + fES(14, 6, z.real()) + fES(14, 6, z.imag()));
      }
      for (int p = 0; p < nfp; ++p) {
        const double* xp = c->xfp.data() + 3 * (size_t)p;
        const bool below = std::fabs(xp[2]) > 1.e-6;
        const std::complex<double> pot = incident_potential(c, k, xp[0], xp[1], xp[2], beta, g);
        const bool sp = special(c->tp[k]);
        const std::complex<double> iw(0.0, c->w1[k]);
        const std::complex<double> vcp = below ? (sp ? rho * pot : iw * rho * pot) : (sp ? pot : iw / g * pot);
        const auto z = wamit_nondim(vcp, below, true, 0, c->tp[k], c->w1[k], c->refl, rho, g);
        const double rel = z.real(), img = z.imag();
        finc.line(hb + fI(10, p + 1) + fES(14, 6, std::abs(z)) + fES(14, 6, std::atan2(img, rel) * (180.0 / kPi)) +
                  fES(14, 6, rel) + fES(14, 6, img));
      }
    }
  }
}

void run(hg_case* c, const char* output_dir, const hg_opts* opts, int nslots) {
  hg_opts o;
  if (opts) o = *opts;
  else hg_default_opts(&o);
  o.solver = c->isolv;  // the deck's Solver_type (ISOLV) picks the linear solver
  hg_ctx* ctx = nullptr;
  int rc = hg_create(&ctx, &o);
  if (rc) raise(rc, "hg_create failed (%d): no usable CUDA device?", rc);
  struct Guard {
    hg_ctx* x;
    ~Guard() { hg_destroy(x); }
  } guard{ctx};
  auto check = [&](int r, const char* what) {
    if (r) raise(r, "%s: %s", what, hg_last_error(ctx));
  };
  check(hg_set_mesh(ctx, c->n, c->ntnd, c->nodes.data(), c->ncon.data(), c->ncn.data(), c->xyz_p.data(), c->ds.data(),
                    c->pnsz.data(), c->dxyz.data(), c->nl, c->nl ? c->lid.data() : nullptr, c->nbody,
                    c->ranges.data()),
        "hg_set_mesh");
  const int np = c->nper, nd = 6 * c->nbody, nbeta = (int)c->headings.size();
  const bool fin = c->h > 0.0;
  const double h = fin ? c->h : -1.0;
  std::vector<double> betas(nbeta);
  for (int i = 0; i < nbeta; ++i) betas[i] = c->headings[i] * kPi / 180.0;
  std::vector<double> amas((size_t)np * nd * nd), bdmp((size_t)np * nd * nd), exfc((size_t)np * 2 * std::max(nbeta, 1) * nd);
  const int nfp = (int)(c->xfp.size() / 3);
  const bool field = nfp > 0;
  std::vector<double> pe;  // per frequency: nfp x (6 nbody + nbeta) COMPLEX*16 (pressure below the surface, elevation on it)
  if (!field) {
    check(hg_solve_sweep(ctx, np, c->v.data(), c->wk.data(), c->w1.data(), h, fin ? c->wvn.data() : nullptr,
                         fin ? kNk : 0, c->irsp, betas.data(), nbeta, c->isol, nslots, amas.data(), bdmp.data(),
                         exfc.data(), nullptr, 0, nullptr),
          "hg_solve_sweep");
  } else {
    const int nc = nd + nbeta;
    pe.assign((size_t)np * nfp * nc * 2, 0.0);
    std::vector<double> prs((size_t)nfp * nc * 2), elv((size_t)nfp * nc * 2);
    for (int k = 0; k < np; ++k) {
      check(hg_solve_frequency(ctx, c->v[k], c->wk[k], c->w1[k], h, fin ? c->wvn.data() + (size_t)k * kNk : nullptr,
                               fin ? kNk : 0, c->irsp, betas.data(), nbeta, c->isol, amas.data() + (size_t)k * nd * nd,
                               bdmp.data() + (size_t)k * nd * nd, exfc.data() + (size_t)k * 2 * nbeta * nd, nullptr, 0),
            "hg_solve_frequency");
      check(hg_field_points(ctx, nfp, c->xfp.data(), 1, c->isol, prs.data(), nfp), "hg_field_points (pressure)");
      check(hg_field_points(ctx, nfp, c->xfp.data(), 2, c->isol, elv.data(), nfp), "hg_field_points (elevation)");
      for (int p = 0; p < nfp; ++p) {
        const bool below = std::fabs(c->xfp[3 * (size_t)p + 2]) > 1.e-6;
        const std::vector<double>& src = below ? prs : elv;
        for (int q = 0; q < nc; ++q)
          for (int r = 0; r < 2; ++r)
            pe[(((size_t)k * nfp + p) * nc + q) * 2 + r] = src[2 * (p + (size_t)q * nfp) + r];
      }
    }
  }
  write_results(c, output_dir, amas.data(), bdmp.data(), exfc.data(), o.rho, o.g);
  if (field && c->nbody > 1) write_pe_multi(c, output_dir, pe, o.rho, o.g);
  if (field && c->nbody == 1) {
    // PressureElevation.6p (formats 1000: ES14.6,I10,12ES14.6 and 1020: 2ES14.6,I10,4ES14.6)
    Out f6(std::string(output_dir) + "/Wamit_format/PressureElevation.6p");
    const int nc = 6 + nbeta;
    for (int k = 0; k < np; ++k) {
      auto val = [&](int p, int q) {
        const double* s = pe.data() + (((size_t)k * nfp + p) * nc + q) * 2;
        return std::complex<double>(s[0], s[1]);
      };
      for (int p = 0; p < nfp; ++p) {
        const bool below = std::fabs(c->xfp[3 * (size_t)p + 2]) > 1.e-6;
        if (!below) continue;
        std::string s = fES(14, 6, c->oufr[k]) + fI(10, p + 1);
        for (int md = 1; md <= 6; ++md) {
          const auto z = wamit_nondim(val(p, md - 1), true, false, md, c->tp[k], c->w1[k], c->refl, o.rho, o.g);
          s += fES(14, 6, z.real()) + fES(14, 6, z.imag());
        }
        f6.line(s);
      }
      for (int ib = 0; ib < nbeta; ++ib) {
        const double beta = c->headings[ib] * kPi / 180.0;
        for (int p = 0; p < nfp; ++p) {
          const bool below = std::fabs(c->xfp[3 * (size_t)p + 2]) > 1.e-6;
          const auto z = wamit_nondim(val(p, 6 + ib), below, true, 0, c->tp[k], c->w1[k], c->refl, o.rho, o.g);
          const double rel = z.real(), img = z.imag();
          f6.line(fES(14, 6, c->oufr[k]) + fES(14, 6, beta * 180.0 / kPi) + fI(10, p + 1) + fES(14, 6, std::abs(z)) +
                  fES(14, 6, std::atan2(img, rel) * (180.0 / kPi)) + fES(14, 6, rel) + fES(14, 6, img));
        }
      }
    }
  }
}

int set_err(char* err, int errlen, const std::string& msg) {
  if (err && errlen > 0) {
    std::strncpy(err, msg.c_str(), (size_t)errlen - 1);
    err[errlen - 1] = '\0';
  }
  return 0;
}

}  // namespace

extern "C" {

int hg_case_read(const char* input_dir, hg_case** out, char* err, int errlen) {
  if (!out) return -1;
  *out = nullptr;
  if (!input_dir) {
    set_err(err, errlen, "input_dir is NULL");
    return -1;
  }
  hg_case* c = new hg_case;
  c->dir = input_dir;
  try {
    read_control(c);
    read_meshes(c);
    read_hydrostatics(c);
    wave_properties(c);
  } catch (const CaseError& e) {
    set_err(err, errlen, e.msg);
    delete c;
    return e.code;
  }
  *out = c;
  return 0;
}

void hg_case_free(hg_case* c) { delete c; }

int hg_case_info(const hg_case* c, int* info, double* dinfo) {
  if (!c || !info) return -1;
  info[0] = c->n;
  info[1] = c->nl;
  info[2] = c->ntnd;
  info[3] = c->nbody;
  info[4] = c->nper;
  info[5] = (int)c->headings.size();
  info[6] = c->irsp;
  info[7] = c->isol;
  info[8] = (int)(c->xfp.size() / 3);
  info[9] = c->sybo;
  info[10] = c->inft;
  info[11] = c->ouft;
  if (dinfo) {
    dinfo[0] = c->h;
    dinfo[1] = c->refl;
  }
  return 0;
}

int hg_case_options(const hg_case* c, int* isolv, int* separate) {
  if (!c) return -1;
  if (isolv) *isolv = c->isolv;
  if (separate) *separate = c->sep ? 1 : 0;
  return 0;
}

int hg_case_arrays(const hg_case* c, double* nodes, int* ncon, int* ncn, double* xyz_p, double* ds, double* pnsz,
                   double* dxyz_p, double* lid_xyz_p, int* body_ranges, double* freq, double* headings) {
  if (!c) return -1;
  auto cp = [](auto* dst, const auto& src) {
    if (dst && !src.empty()) std::copy(src.begin(), src.end(), dst);
  };
  cp(nodes, c->nodes);
  cp(ncon, c->ncon);
  cp(ncn, c->ncn);
  cp(xyz_p, c->xyz_p);
  cp(ds, c->ds);
  cp(pnsz, c->pnsz);
  cp(dxyz_p, c->dxyz);
  cp(lid_xyz_p, c->lid);
  cp(body_ranges, c->ranges);
  if (freq)
    for (int k = 0; k < c->nper; ++k) {
      freq[6 * k + 0] = c->v[k];
      freq[6 * k + 1] = c->wk[k];
      freq[6 * k + 2] = c->w1[k];
      freq[6 * k + 3] = c->tp[k];
      freq[6 * k + 4] = c->wl[k];
      freq[6 * k + 5] = c->oufr[k];
    }
  cp(headings, c->headings);
  return 0;
}

int hg_case_write(const hg_case* c, const char* output_dir, const double* amas, const double* bdmp, const double* exfc,
                  double rho, double g, char* err, int errlen) {
  if (!c || !output_dir || !amas || !bdmp || !exfc) {
    set_err(err, errlen, "NULL argument");
    return -1;
  }
  try {
    write_results(c, output_dir, amas, bdmp, exfc, rho, g);
  } catch (const CaseError& e) {
    set_err(err, errlen, e.msg);
    return e.code;
  }
  return 0;
}

int hg_case_run(hg_case* c, const char* output_dir, const hg_opts* opts, int nslots, char* err, int errlen) {
  if (!c || !output_dir) {
    set_err(err, errlen, "NULL argument");
    return -1;
  }
  if (nslots < 1 || nslots > 16) {
    set_err(err, errlen, "nslots must be in 1..16");
    return -4;
  }
  try {
    run(c, output_dir, opts, nslots);
  } catch (const CaseError& e) {
    set_err(err, errlen, e.msg);
    return e.code;
  }
  return 0;
}

}  // extern "C"
