// Host side of the wavefunction model: wfx parsing, primitive pruning,
// cutoffs and ordering, molecular cell.  Mirrors critic2's molwfn set-up
// (src/wfn_private@proc.F90:1121-1284, 3632-3785 and
// src/crystalmod@proc.f90:222-249, 545).
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <numeric>
#include <sstream>

#include "c2g_internal.h"

namespace c2g {

const int kLi[56][3] = {
    {0, 0, 0},
    {1, 0, 0}, {0, 1, 0}, {0, 0, 1},
    {2, 0, 0}, {0, 2, 0}, {0, 0, 2}, {1, 1, 0}, {1, 0, 1}, {0, 1, 1},
    {3, 0, 0}, {0, 3, 0}, {0, 0, 3}, {2, 1, 0}, {2, 0, 1}, {0, 2, 1},
    {1, 2, 0}, {1, 0, 2}, {0, 1, 2}, {1, 1, 1},
    {4, 0, 0}, {0, 4, 0}, {0, 0, 4}, {3, 1, 0}, {3, 0, 1}, {1, 3, 0}, {0, 3, 1}, {1, 0, 3},
    {0, 1, 3}, {2, 2, 0}, {2, 0, 2}, {0, 2, 2}, {2, 1, 1}, {1, 2, 1}, {1, 1, 2},
    {0, 0, 5}, {0, 1, 4}, {0, 2, 3}, {0, 3, 2}, {0, 4, 1}, {0, 5, 0}, {1, 0, 4}, {1, 1, 3},
    {1, 2, 2}, {1, 3, 1}, {1, 4, 0}, {2, 0, 3}, {2, 1, 2}, {2, 2, 1}, {2, 3, 0}, {3, 0, 2},
    {3, 1, 1}, {3, 2, 0}, {4, 0, 1}, {4, 1, 0}, {5, 0, 0}};

static const double kPrimThreshold = 1e-12;          // rprim_thres
static const double kBorder = 10.0 / 0.52917720859;  // rborder_def (bohr)

// Merge primitives with equal exponent (1e-12), type and centre, summing
// their coefficient columns; survivors keep their original relative order.
void prune_primitives(HostWfn &w) {
  const int n = w.npri, nmo = w.nmo;
  std::vector<int> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return w.e[a] < w.e[b]; });
  std::vector<char> keep(n, 1);
  for (int i = 0; i < n; i++) {
    const int a = order[i];
    if (!keep[a]) continue;
    for (int j = i + 1; j < n; j++) {
      const int b = order[j];
      if (std::fabs(w.e[b] - w.e[a]) > 1e-12) continue;
      if (keep[b] && w.itype[a] == w.itype[b] && w.icenter[a] == w.icenter[b]) {
        double *ca = &w.cmo[(size_t)a * nmo];
        const double *cb = &w.cmo[(size_t)b * nmo];
        for (int m = 0; m < nmo; m++) ca[m] += cb[m];
        keep[b] = 0;
      }
    }
  }
  int j = 0;
  for (int i = 0; i < n; i++) {
    if (!keep[i]) continue;
    if (i != j) {
      std::copy(w.cmo.begin() + (size_t)i * nmo, w.cmo.begin() + (size_t)(i + 1) * nmo,
                w.cmo.begin() + (size_t)j * nmo);
      w.e[j] = w.e[i];
      w.icenter[j] = w.icenter[i];
      w.itype[j] = w.itype[i];
    }
    j++;
  }
  w.npri = j;
  w.e.resize(j);
  w.icenter.resize(j);
  w.itype.resize(j);
  w.cmo.resize((size_t)j * nmo);
}

void complete_struct(HostWfn &w) {
  w.dran.assign(w.npri, 0.0);
  w.spcutoff.assign(w.natom, 0.0);
  w.lmax.assign(w.natom, 0);
  for (int i = 0; i < w.npri; i++) {
    w.dran[i] = std::sqrt(-std::log(kPrimThreshold) / w.e[i]);
    const int a = w.icenter[i];
    w.spcutoff[a] = std::max(w.spcutoff[a], w.dran[i]);
    const int *l = kLi[w.itype[i] - 1];
    w.lmax[a] = std::max(w.lmax[a], std::max(l[0], std::max(l[1], l[2])));
  }
  w.icord.resize(w.npri);
  std::iota(w.icord.begin(), w.icord.end(), 0);
  std::stable_sort(w.icord.begin(), w.icord.end(),
                   [&](int a, int b) { return w.icenter[a] < w.icenter[b]; });
  w.iprilo.assign(w.natom, 0);
  w.iprihi.assign(w.natom, -1);
  std::vector<char> seen(w.natom, 0);
  for (int k = 0; k < w.npri; k++) {
    const int a = w.icenter[w.icord[k]];
    if (!seen[a]) w.iprilo[a] = k, seen[a] = 1;
    w.iprihi[a] = k;
  }
  // EDF cutoffs widen the atoms' environment radius (:3750-3756)
  w.edf_dran.assign(w.nedf, 0.0);
  for (int i = 0; i < w.nedf; i++) {
    w.edf_dran[i] = std::sqrt(-std::log(kPrimThreshold) / w.edf_e[i]);
    const int a = w.edf_icenter[i];
    w.spcutoff[a] = std::max(w.spcutoff[a], w.edf_dran[i]);
  }
}

void molecular_cell(HostWfn &w) {
  for (int j = 0; j < 3; j++) {
    double lo = 1e40, hi = -1e40;
    for (int a = 0; a < w.natom; a++) {
      lo = std::min(lo, w.xyz[3 * a + j] - kBorder);
      hi = std::max(hi, w.xyz[3 * a + j] + kBorder);
    }
    w.cell_lo[j] = lo;
    w.cell_aa[j] = hi - lo;
    w.molborder[j] = std::max(kBorder - std::max(2.0, 0.8 * kBorder), 0.0) / (hi - lo);
  }
}

// ------------------------------------------------------------------ wfx
namespace {

std::string trim(const std::string &s) {
  size_t a = 0, b = s.size();
  while (a < b && std::isspace((unsigned char)s[a])) a++;
  while (b > a && std::isspace((unsigned char)s[b - 1])) b--;
  return s.substr(a, b - a);
}

// Reads whitespace-separated numbers until a line starting with '<'
// (the way critic2's wfx_read_* helpers end a block).
template <class T>
bool read_block(std::istream &in, std::vector<T> &out, size_t n, std::string *stop) {
  out.clear();
  std::string line;
  while (std::getline(in, line)) {
    std::string t = trim(line);
    if (!t.empty() && t[0] == '<') {
      if (stop) *stop = t;
      break;
    }
    std::istringstream ss(t);
    std::string tok;
    while (ss >> tok) {
      for (char &c : tok)
        if (c == 'D' || c == 'd') c = 'E';
      char *end = nullptr;
      double v = std::strtod(tok.c_str(), &end);
      if (end == tok.c_str()) return false;
      out.push_back((T)v);
    }
  }
  return out.size() == n;
}

}  // namespace

bool read_wfx(const char *path, HostWfn &w, std::string &err) {
  std::ifstream in(path);
  if (!in) {
    err = std::string("cannot open ") + path;
    return false;
  }
  // first pass: sizes
  int nat = 0, nmo = 0, npri = 0, nalpha = 0, nedf = 0;
  std::string line;
  auto next_int = [&](int &v) {
    std::string l2;
    if (!std::getline(in, l2)) return false;
    v = std::atoi(trim(l2).c_str());
    return true;
  };
  while (std::getline(in, line)) {
    std::string t = trim(line);
    if (t == "<Number of Nuclei>") next_int(nat);
    else if (t == "<Number of Occupied Molecular Orbitals>") next_int(nmo);
    else if (t == "<Number of Primitives>") next_int(npri);
    else if (t == "<Number of Alpha Electrons>") next_int(nalpha);
    else if (t == "<Number of EDF Primitives>") next_int(nedf);
  }
  if (nmo <= 0) { err = "Number of Occupied Molecular Orbitals tag not found"; return false; }
  if (npri <= 0) { err = "Number of Primitives tag not found"; return false; }
  if (nat <= 0) { err = "Number of Nuclei tag not found"; return false; }
  in.clear();
  in.seekg(0);
  w = HostWfn();
  w.natom = nat;
  w.npri = npri;
  w.nmo = nmo;
  w.cmo.assign((size_t)npri * nmo, 0.0);
  w.nedf = std::max(nedf, 0);
  std::vector<double> buf;
  bool have_xyz = false, have_z = false, have_c = false, have_t = false, have_e = false,
       have_o = false, have_mo = false;
  int have_edf = 0;  // bit per EDF section: centres, types, exponents, coefficients
  while (std::getline(in, line)) {
    std::string t = trim(line);
    if (t.size() < 2 || t[0] != '<' || t[1] == '/') continue;
    if (t == "<Atomic Numbers>") {
      if (!read_block(in, buf, nat, nullptr)) { err = "bad <Atomic Numbers>"; return false; }
      w.z.assign(buf.begin(), buf.end());
      have_z = true;
    } else if (t == "<Nuclear Cartesian Coordinates>") {
      if (!read_block(in, buf, 3 * (size_t)nat, nullptr)) { err = "bad coordinates"; return false; }
      w.xyz = buf;
      have_xyz = true;
    } else if (t == "<Primitive Centers>") {
      if (!read_block(in, buf, npri, nullptr)) { err = "bad <Primitive Centers>"; return false; }
      w.icenter.resize(npri);
      for (int i = 0; i < npri; i++) w.icenter[i] = (int)buf[i] - 1;
      have_c = true;
    } else if (t == "<Primitive Types>") {
      if (!read_block(in, buf, npri, nullptr)) { err = "bad <Primitive Types>"; return false; }
      w.itype.assign(buf.begin(), buf.end());
      for (int v : w.itype)
        if (v < 1 || v > 56) { err = "primitive type not supported"; return false; }
      have_t = true;
    } else if (t == "<Primitive Exponents>") {
      if (!read_block(in, w.e, npri, nullptr)) { err = "bad <Primitive Exponents>"; return false; }
      have_e = true;
    } else if (t == "<Molecular Orbital Occupation Numbers>") {
      if (!read_block(in, w.occ, nmo, nullptr)) { err = "bad occupations"; return false; }
      have_o = true;
    } else if (t == "<Molecular Orbital Primitive Coefficients>") {
      // <MO Number> / i / </MO Number> / coefficients, repeated
      std::string l2;
      std::getline(in, l2);  // <MO Number>
      for (int m = 0; m < nmo; m++) {
        std::getline(in, l2);  // MO index
        std::getline(in, l2);  // </MO Number>
        std::string stop;
        if (!read_block(in, buf, npri, &stop)) { err = "bad MO coefficients"; return false; }
        for (int i = 0; i < npri; i++) w.cmo[(size_t)i * nmo + m] = buf[i];
      }
      have_mo = true;
    } else if (w.nedf > 0 && t == "<EDF Primitive Centers>") {
      if (!read_block(in, buf, w.nedf, nullptr)) { err = "bad <EDF Primitive Centers>"; return false; }
      w.edf_icenter.resize(w.nedf);
      for (int i = 0; i < w.nedf; i++) w.edf_icenter[i] = (int)buf[i] - 1;
      have_edf |= 1;
    } else if (w.nedf > 0 && t == "<EDF Primitive Types>") {
      if (!read_block(in, buf, w.nedf, nullptr)) { err = "bad <EDF Primitive Types>"; return false; }
      w.edf_itype.assign(buf.begin(), buf.end());
      for (int v : w.edf_itype)
        if (v < 1 || v > 56) { err = "primitive type not supported"; return false; }
      have_edf |= 2;
    } else if (w.nedf > 0 && t == "<EDF Primitive Exponents>") {
      if (!read_block(in, w.edf_e, w.nedf, nullptr)) { err = "bad <EDF Primitive Exponents>"; return false; }
      have_edf |= 4;
    } else if (w.nedf > 0 && t == "<EDF Primitive Coefficients>") {
      if (!read_block(in, w.edf_c, w.nedf, nullptr)) { err = "bad <EDF Primitive Coefficients>"; return false; }
      have_edf |= 8;
    }
  }
  if (w.nedf > 0 && have_edf != 15) {
    err = "wfx file is missing an EDF section";
    return false;
  }
  for (int i = 0; i < w.nedf; i++) {
    if (w.edf_icenter[i] < 0 || w.edf_icenter[i] >= nat) { err = "EDF primitive centre out of range"; return false; }
    if (!(w.edf_e[i] > 0.0)) { err = "EDF exponents must be positive"; return false; }
  }
  if (!(have_xyz && have_z && have_c && have_t && have_e && have_o && have_mo)) {
    err = "wfx file is missing a required section";
    return false;
  }
  for (int i = 0; i < npri; i++)
    if (w.icenter[i] < 0 || w.icenter[i] >= nat) { err = "primitive centre out of range"; return false; }
  // wavefunction type from the occupations (src/wfn_private@proc.F90:1240-1268)
  bool frac = false;
  int n1 = 0, n2 = 0;
  for (double o : w.occ) {
    long io = std::lround(o);
    if (std::fabs((double)io - o) > 1e-10) frac = true;
    else if (io == 1) n1++;
    else if (io == 2) n2++;
  }
  if (frac) w.wfntyp = C2G_WFN_FRAC, w.nalpha = 0;
  else if (n1 == 0) w.wfntyp = C2G_WFN_RHF, w.nalpha = nalpha;
  else if (n2 == 0) w.wfntyp = C2G_WFN_UHF, w.nalpha = nalpha;
  else w.wfntyp = C2G_WFN_ROHF, w.nalpha = n2;
  prune_primitives(w);
  complete_struct(w);
  molecular_cell(w);
  return true;
}

// ------------------------------------------------------------------ wfn
namespace {

// Element symbols by atomic number (index 0 unused).
const char *const kElem[] = {
    "",   "H",  "He", "Li", "Be", "B",  "C",  "N",  "O",  "F",  "Ne", "Na", "Mg", "Al", "Si", "P",  "S",
    "Cl", "Ar", "K",  "Ca", "Sc", "Ti", "V",  "Cr", "Mn", "Fe", "Co", "Ni", "Cu", "Zn", "Ga", "Ge", "As",
    "Se", "Br", "Kr", "Rb", "Sr", "Y",  "Zr", "Nb", "Mo", "Tc", "Ru", "Rh", "Pd", "Ag", "Cd", "In", "Sn",
    "Sb", "Te", "I",  "Xe", "Cs", "Ba", "La", "Ce", "Pr", "Nd", "Pm", "Sm", "Eu", "Gd", "Tb", "Dy", "Ho",
    "Er", "Tm", "Yb", "Lu", "Hf", "Ta", "W",  "Re", "Os", "Ir", "Pt", "Au", "Hg", "Tl", "Pb", "Bi", "Po",
    "At", "Rn", "Fr", "Ra", "Ac", "Th", "Pa", "U",  "Np", "Pu", "Am", "Cm", "Bk", "Cf", "Es", "Fm", "Md",
    "No", "Lr", "Rf", "Db", "Sg", "Bh", "Hs", "Mt", "Ds", "Rg", "Cn", "Nh", "Fl", "Mc", "Lv", "Ts", "Og"};

// Atomic number from a label such as "C", "Cl", "c12", "CL" (the role of
// zatguess, src/tools_io@proc.f90): the letters at the start, a two-letter
// symbol first, then one letter; 0 when nothing matches.
int zatguess(const std::string &label) {
  std::string l;
  for (char c : label) {
    if (std::isalpha((unsigned char)c)) l += c;
    else if (!l.empty()) break;
  }
  if (l.empty()) return 0;
  auto match = [&](const std::string &sym) {
    for (int z = 1; z < (int)(sizeof(kElem) / sizeof(kElem[0])); z++) {
      const char *e = kElem[z];
      if (std::strlen(e) != sym.size()) continue;
      bool ok = true;
      for (size_t i = 0; i < sym.size(); i++)
        ok = ok && std::tolower((unsigned char)e[i]) == std::tolower((unsigned char)sym[i]);
      if (ok) return z;
    }
    return 0;
  };
  if (l.size() >= 2) {
    const int z = match(l.substr(0, 2));
    if (z) return z;
  }
  return match(l.substr(0, 1));
}

// Fortran formatted input of one real field (Fw.d / Ew.d): blanks ignored,
// D or E exponent (or a signed exponent without the letter), and d implied
// decimals when the field has no point.  An all-blank field reads as 0.
bool fortran_real(const std::string &field, int d, double &v) {
  std::string t;
  for (char c : field)
    if (c != ' ') t += c;
  v = 0.0;
  if (t.empty()) return true;
  size_t epos = std::string::npos;
  for (size_t i = 1; i < t.size(); i++) {
    const char c = t[i];
    if (c == 'D' || c == 'd' || c == 'E' || c == 'e' || c == 'Q' || c == 'q') { epos = i; break; }
    if ((c == '+' || c == '-') && t[i - 1] != 'e' && t[i - 1] != 'E' && t[i - 1] != 'd' && t[i - 1] != 'D') {
      epos = i;
      break;
    }
  }
  std::string mant = t.substr(0, epos), ex;
  if (epos != std::string::npos) ex = t.substr(t[epos] == '+' || t[epos] == '-' ? epos : epos + 1);
  char *end = nullptr;
  std::strtod(mant.c_str(), &end);
  if (end == mant.c_str() || *end != '\0') return false;
  long e10 = 0;
  if (!ex.empty()) {
    e10 = std::strtol(ex.c_str(), &end, 10);
    if (end == ex.c_str() || *end != '\0') return false;
  }
  if (mant.find('.') == std::string::npos) e10 -= d;
  // one correctly rounded conversion of mantissa and exponent together
  const std::string full = mant + "e" + std::to_string(e10);
  v = std::strtod(full.c_str(), &end);
  return *end == '\0';
}

bool fortran_int(const std::string &field, long &v) {
  std::string t;
  for (char c : field)
    if (c != ' ') t += c;
  v = 0;
  if (t.empty()) return true;
  char *end = nullptr;
  v = std::strtol(t.c_str(), &end, 10);
  return end != t.c_str() && *end == '\0';
}

// Columns [a, a + w) (0-based) of a record padded with blanks.
std::string col(const std::string &line, size_t a, size_t w) {
  std::string r = a < line.size() ? line.substr(a, w) : std::string();
  r.resize(w, ' ');
  return r;
}

// Reads n fixed-width fields of a repeated format (skip columns, then up to
// per fields of width w per record), continuing on new records as Fortran's
// format reversion does.
template <class F>
bool read_fields(std::istream &in, size_t n, size_t skip, size_t per, size_t w, F &&put) {
  size_t got = 0;
  std::string line;
  while (got < n) {
    if (!std::getline(in, line)) return false;
    if (!line.empty() && line.back() == '\r') line.pop_back();
    for (size_t k = 0; k < per && got < n; k++, got++)
      if (!put(got, col(line, skip + k * w, w))) return false;
  }
  return true;
}

}  // namespace

// read_wfn (src/wfn_private@proc.F90:981-1118): the AIMPAC wfn format with
// its fixed columns (formats 101-106 there): header (MO, primitive and
// nucleus counts), nuclei, centre and type assignments, exponents, any ECP
// lines up to the first MO record, then per MO its occupation, energy and
// coefficients.  The wavefunction type follows from the occupations, and a
// UHF file's alpha count from the first drop of the orbital energy.
bool read_wfn(const char *path, HostWfn &w, std::string &err) {
  std::ifstream in(path);
  if (!in) {
    err = std::string("cannot open ") + path;
    return false;
  }
  err = std::string("Error reading file: ") + path;
  std::string line;
  if (!std::getline(in, line) || !std::getline(in, line)) return false;
  if (!line.empty() && line.back() == '\r') line.pop_back();
  long nmo = 0, npri = 0, nat = 0;
  if (!fortran_int(col(line, 18, 5), nmo) || !fortran_int(col(line, 38, 5), npri) ||
      !fortran_int(col(line, 58, 5), nat))
    return false;
  if (nmo <= 0 || npri <= 0 || nat <= 0) return false;
  w = HostWfn();
  w.natom = (int)nat, w.npri = (int)npri, w.nmo = (int)nmo;
  w.xyz.resize(3 * nat);
  w.z.resize(nat);
  for (long a = 0; a < nat; a++) {
    if (!std::getline(in, line)) return false;
    if (!line.empty() && line.back() == '\r') line.pop_back();
    for (int j = 0; j < 3; j++)
      if (!fortran_real(col(line, 24 + 12 * j, 12), 8, w.xyz[3 * a + j])) return false;
    w.z[a] = zatguess(col(line, 2, 2));
    if (w.z[a] == 0) {
      err = "unknown element in " + std::string(path);
      return false;
    }
  }
  w.icenter.resize(npri);
  w.itype.resize(npri);
  w.e.resize(npri);
  if (!read_fields(in, npri, 20, 20, 3, [&](size_t i, const std::string &f) {
        long v;
        if (!fortran_int(f, v)) return false;
        w.icenter[i] = (int)v - 1;
        return true;
      }))
    return false;
  if (!read_fields(in, npri, 20, 20, 3, [&](size_t i, const std::string &f) {
        long v;
        if (!fortran_int(f, v)) return false;
        w.itype[i] = (int)v;
        return true;
      }))
    return false;
  for (int v : w.itype)
    if (v < 1 || v > 56) {
      err = "primitive type not supported";
      return false;
    }
  for (int v : w.icenter)
    if (v < 0 || v >= nat) return false;
  if (!read_fields(in, npri, 10, 5, 14, [&](size_t i, const std::string &f) { return fortran_real(f, 7, w.e[i]); }))
    return false;
  // skip ECP records up to the first one that starts with "MO"
  std::streampos pos;
  for (;;) {
    pos = in.tellg();
    if (!std::getline(in, line)) return false;
    if (line.size() >= 2 && line[0] == 'M' && line[1] == 'O') break;
  }
  in.seekg(pos);
  w.occ.resize(nmo);
  w.cmo.assign((size_t)npri * nmo, 0.0);
  bool frac = false, found = false;
  int n1 = 0, n2 = 0, nalpha = -1;
  double ene0 = -1e30;
  for (long m = 0; m < nmo; m++) {
    if (!std::getline(in, line)) return false;
    if (!line.empty() && line.back() == '\r') line.pop_back();
    double ene = 0.0;
    if (!fortran_real(col(line, 35, 12), 7, w.occ[m]) || !fortran_real(col(line, 62, 12), 6, ene)) return false;
    if (!read_fields(in, npri, 0, 5, 16, [&](size_t i, const std::string &f) {
          return fortran_real(f, 8, w.cmo[i * nmo + m]);
        }))
      return false;
    const long io = std::lround(w.occ[m]);
    if (std::fabs((double)io - w.occ[m]) > 1e-10) frac = true;
    else if (io == 1) n1++;
    else if (io == 2) n2++;
    if (ene < ene0 - 1e-3) nalpha = (int)m, found = true;
    ene0 = ene;
  }
  if (frac) w.wfntyp = C2G_WFN_FRAC, w.nalpha = 0;
  else if (n1 == 0) w.wfntyp = C2G_WFN_RHF, w.nalpha = nalpha;
  else if (n2 == 0) w.wfntyp = C2G_WFN_UHF, w.nalpha = found ? nalpha : (int)nmo;
  else w.wfntyp = C2G_WFN_ROHF, w.nalpha = n2;
  err.clear();
  prune_primitives(w);
  complete_struct(w);
  molecular_cell(w);
  return true;
}

}  // namespace c2g
