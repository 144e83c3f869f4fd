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
#include "sphcar_tables.h"

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

// ----------------------------------------------------------------- fchk
namespace {

// Normalisation of a Cartesian primitive x^a y^b z^c exp(-al r^2) (gnorm,
// src/wfn_private@proc.F90:3375-3459, in closed form).
double gnorm_cart(const int *l, double al) {
  const int L = l[0] + l[1] + l[2];
  double df = 1.0;
  for (int k = 0; k < 3; k++)
    for (int v = 2 * l[k] - 1; v > 1; v -= 2) df *= v;
  return std::pow(2.0, (4.0 * L + 3.0) / 4.0) * std::pow(al, (2.0 * L + 3.0) / 4.0) /
         std::pow(M_PI, 0.75) / std::sqrt(df);
}

// Normalisation of a contracted Cartesian function with coefficients c of
// normalised primitives (aonorm, :3461-3540).
double aonorm_cart(const int *l, int n, const double *a, const double *c) {
  const int L = l[0] + l[1] + l[2];
  double df = 1.0;
  for (int k = 0; k < 3; k++)
    for (int v = 2 * l[k] - 1; v > 1; v -= 2) df *= v;
  double s = 0.0;
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) s += c[i] * c[j] / std::pow(a[i] + a[j], L + 1.5);
  s *= df * std::pow(M_PI, 1.5) / std::pow(2.0, L);
  return 1.0 / std::sqrt(s);
}

// fchk Cartesian components of a shell of angular momentum l, as critic2
// li types (the order of Gaussian's checkpoint files)
std::vector<int> fchk_cart_types(int l) {
  static const char *const ord[5][15] = {
      {"", 0},
      {"x", "y", "z"},
      {"xx", "yy", "zz", "xy", "xz", "yz"},
      {"xxx", "yyy", "zzz", "xyy", "xxy", "xxz", "xzz", "yzz", "yyz", "xyz"},
      {"zzzz", "yzzz", "yyzz", "yyyz", "yyyy", "xzzz", "xyzz", "xyyz", "xyyy", "xxzz", "xxyz", "xxyy", "xxxz",
       "xxxy", "xxxx"}};
  static const int n[5] = {1, 3, 6, 10, 15};
  std::vector<int> t;
  for (int i = 0; i < n[l]; i++) {
    int e[3] = {0, 0, 0};
    for (const char *c = ord[l][i]; c && *c; c++) e[*c - 'x']++;
    for (int k = 0; k < 56; k++)
      if (kLi[k][0] == e[0] && kLi[k][1] == e[1] && kLi[k][2] == e[2]) {
        t.push_back(k + 1);
        break;
      }
  }
  return t;
}

}  // namespace

// read_fchk (src/wfn_private@proc.F90:1287-1812) without virtual orbitals:
// the occupied MOs of a Gaussian formatted checkpoint, sp shells unfolded,
// pure d/f/g shells transformed to Cartesian Gaussians (real solid
// harmonics in Gaussian's m = 0, 1, -1, ... order), every Cartesian
// component normalised with its own primitive and contraction factors.
bool read_fchk(const char *path, HostWfn &w, std::string &err) {
  std::ifstream in(path);
  if (!in) {
    err = std::string("cannot open ") + path;
    return false;
  }
  err = std::string("Error reading file: ") + path;
  std::vector<std::string> lines;
  for (std::string l; std::getline(in, l);) {
    if (!l.empty() && l.back() == '\r') l.pop_back();
    lines.push_back(l);
  }
  auto starts = [](const std::string &l, const char *key) { return l.compare(0, std::strlen(key), key) == 0; };
  auto last_int = [](const std::string &l, long &v) {
    std::istringstream ss(l);
    std::string tok, lastt;
    while (ss >> tok) lastt = tok;
    char *end = nullptr;
    v = std::strtol(lastt.c_str(), &end, 10);
    return end != lastt.c_str() && *end == '\0';
  };
  long nelec = 0, nalpha = 0, nbeta = 0, nbas = 0, ncshel = 0, nshel = 0, natom = 0, nmoa = 0;
  bool uhf = false;
  for (const std::string &l : lines) {
    long v = 0;
    if (starts(l, "Number of electrons") && last_int(l, v)) nelec = v;
    else if (starts(l, "Number of alpha electrons") && last_int(l, v)) nalpha = v;
    else if (starts(l, "Number of beta electrons") && last_int(l, v)) nbeta = v;
    else if (starts(l, "Number of basis functions") && last_int(l, v)) nbas = v;
    else if (starts(l, "Number of contracted shells") && last_int(l, v)) ncshel = v;
    else if (starts(l, "Number of primitive shells") && last_int(l, v)) nshel = v;
    else if (starts(l, "Atomic numbers") && last_int(l, v)) natom = v;
    else if (starts(l, "Alpha Orbital Energies") && last_int(l, v)) nmoa = v;
    else if (starts(l, "Beta Orbital Energies")) uhf = true;
  }
  if (nelec == 0) { err = "nelec = 0 reading fchk file"; return false; }
  if (nmoa == 0) { err = "nmoall = 0 reading fchk file"; return false; }
  if (ncshel <= 0 || nshel <= 0 || nbas <= 0 || natom <= 0) return false;
  int wfntyp, nmoocc, nalf;
  if (uhf) wfntyp = C2G_WFN_UHF, nmoocc = (int)nelec, nalf = (int)nalpha;
  else if (nalpha == nbeta) wfntyp = C2G_WFN_RHF, nmoocc = (int)(nelec / 2), nalf = (int)(nelec / 2);
  else wfntyp = C2G_WFN_ROHF, nmoocc = (int)nalpha, nalf = (int)nbeta;
  const int namo = wfntyp == C2G_WFN_ROHF ? nmoocc : nalf;  // alpha MOs read
  // array sections: the values after a "Name  X  N=  n" line
  auto section = [&](const char *key, size_t n, std::vector<double> &out) {
    out.clear();
    for (size_t i = 0; i < lines.size(); i++) {
      if (!starts(lines[i], key)) continue;
      for (size_t j = i + 1; j < lines.size() && out.size() < n; j++) {
        std::istringstream ss(lines[j]);
        std::string tok;
        while (out.size() < n && ss >> tok) {
          for (char &c : tok)
            if (c == 'D' || c == 'd') c = 'E';
          char *end = nullptr;
          const double v = std::strtod(tok.c_str(), &end);
          if (end == tok.c_str() || *end != '\0') return false;
          out.push_back(v);
        }
      }
      return out.size() == n;
    }
    return false;
  };
  std::vector<double> zs, xyz, st, np_, sa, ex, cc, pc, moa, mob;
  if (!section("Atomic numbers", natom, zs) || !section("Current cartesian coordinates", 3 * natom, xyz) ||
      !section("Shell types", ncshel, st) || !section("Number of primitives per shell", ncshel, np_) ||
      !section("Shell to atom map", ncshel, sa) || !section("Primitive exponents", nshel, ex) ||
      !section("Contraction coefficients", nshel, cc))
    return false;
  bool has_sp = false;
  for (double t : st) has_sp = has_sp || (int)t == -1;
  if (has_sp && !section("P(S=P) Contraction coefficients", nshel, pc)) return false;
  if (!section("Alpha MO coefficients", (size_t)namo * nbas, moa)) return false;
  if (nmoocc > namo && !section("Beta MO coefficients", (size_t)(nmoocc - namo) * nbas, mob)) return false;
  // unfold sp shells: (type, nprim, atom, exponents, coefficients)
  struct Shell {
    int type, atom;
    std::vector<double> a, c;
  };
  std::vector<Shell> sh;
  size_t off = 0;
  for (long i = 0; i < ncshel; i++) {
    const int t = (int)st[i], n = (int)np_[i], at = (int)sa[i] - 1;
    if (at < 0 || at >= natom || n <= 0) return false;
    std::vector<double> a(ex.begin() + off, ex.begin() + off + n), c(cc.begin() + off, cc.begin() + off + n);
    if (t == -1) {
      sh.push_back({0, at, a, c});
      sh.push_back({1, at, a, std::vector<double>(pc.begin() + off, pc.begin() + off + n)});
    } else {
      sh.push_back({t, at, a, c});
    }
    off += n;
  }
  for (const Shell &s : sh)
    if (std::abs(s.type) > 4) { err = "h primitives not supported in fchk"; return false; }
  auto nsph = [](int t) { return t < 0 ? 2 * (-t) + 1 : (t + 1) * (t + 2) / 2; };
  long nb = 0;
  for (const Shell &s : sh) nb += nsph(s.type);
  if (nb != nbas) { err = "basis function count does not match the shells"; return false; }
  // MO coefficients (MO-major, shell order) -> Cartesian components
  std::vector<const double *> mo(nmoocc);
  for (int m = 0; m < nmoocc; m++)
    mo[m] = m < namo ? moa.data() + (size_t)m * nbas : mob.data() + (size_t)(m - namo) * nbas;
  w = HostWfn();
  w.natom = (int)natom;
  w.nmo = nmoocc;
  w.xyz = xyz;
  w.z.resize(natom);
  for (long a = 0; a < natom; a++) w.z[a] = (int)std::lround(zs[a]);
  std::vector<std::vector<double>> cols;  // per primitive: nmo coefficients
  long ns = 0;
  for (const Shell &s : sh) {
    const int l = std::abs(s.type), ncar = (l + 1) * (l + 2) / 2, nsp = nsph(s.type);
    const std::vector<int> types = fchk_cart_types(l);
    const double *T = l == 2 ? &kSphCar2[0][0] : l == 3 ? &kSphCar3[0][0] : l == 4 ? &kSphCar4[0][0] : nullptr;
    std::vector<double> car((size_t)nmoocc * ncar, 0.0);
    for (int m = 0; m < nmoocc; m++)
      for (int c = 0; c < ncar; c++) {
        if (s.type >= 0 || l < 2) {
          car[(size_t)m * ncar + c] = mo[m][ns + c];
        } else {
          double v = 0.0;
          for (int k = 0; k < nsp; k++) v += mo[m][ns + k] * T[(size_t)k * ncar + c];
          car[(size_t)m * ncar + c] = v;
        }
      }
    const int n = (int)s.a.size();
    for (int c = 0; c < ncar; c++) {
      const int ityp = types[c];
      const int *lv = kLi[ityp - 1];
      std::vector<double> cn(n);
      for (int k = 0; k < n; k++) cn[k] = s.c[k] * gnorm_cart(lv, s.a[k]);
      const double norm = aonorm_cart(lv, n, s.a.data(), cn.data());
      for (int k = 0; k < n; k++) {
        w.icenter.push_back(s.atom);
        w.itype.push_back(ityp);
        w.e.push_back(s.a[k]);
        std::vector<double> col(nmoocc);
        for (int m = 0; m < nmoocc; m++) col[m] = cn[k] * norm * car[(size_t)m * ncar + c];
        cols.push_back(col);
      }
    }
    ns += nsp;
  }
  w.npri = (int)w.e.size();
  w.cmo.resize((size_t)w.npri * nmoocc);
  for (int i = 0; i < w.npri; i++)
    std::copy(cols[i].begin(), cols[i].end(), w.cmo.begin() + (size_t)i * nmoocc);
  w.occ.assign(nmoocc, wfntyp == C2G_WFN_UHF ? 1.0 : 2.0);
  if (wfntyp == C2G_WFN_ROHF)
    for (int m = nalf; m < nmoocc; m++) w.occ[m] = 1.0;
  w.wfntyp = wfntyp;
  w.nalpha = nalf;
  err.clear();
  prune_primitives(w);
  complete_struct(w);
  molecular_cell(w);
  return true;
}

// --------------------------------------------------------------- molden
namespace {

std::string lower_str(std::string s) {
  for (char &c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}

bool parse_real(std::string t, double &v) {
  for (char &c : t)
    if (c == 'D' || c == 'd') c = 'E';
  char *end = nullptr;
  v = std::strtod(t.c_str(), &end);
  return end != t.c_str() && *end == '\0';
}

// molden Cartesian component order of a shell, as critic2 li types
std::vector<int> molden_cart_types(int l) {
  if (l != 4) return fchk_cart_types(l);
  static const char *const g[15] = {"xxxx", "yyyy", "zzzz", "xxxy", "xxxz", "xyyy", "yyyz", "xzzz",
                                    "yzzz", "xxyy", "xxzz", "yyzz", "xxyz", "xyyz", "xyzz"};
  std::vector<int> t;
  for (const char *lab : g) {
    int e[3] = {0, 0, 0};
    for (const char *c = lab; *c; c++) e[*c - 'x']++;
    for (int k = 0; k < 56; k++)
      if (kLi[k][0] == e[0] && kLi[k][1] == e[1] && kLi[k][2] == e[2]) {
        t.push_back(k + 1);
        break;
      }
  }
  return t;
}

}  // namespace

// read_molden (src/wfn_private@proc.F90:1819-2478) for Gaussian-type
// orbitals without virtual orbitals: [Atoms] (AU or Angs), [GTO], the
// [5D]/[5D7F]/[5D10F]/[7F]/[9G] flags, [MO] (occupied MOs, Spin= and
// Occup=).  ORCA files (title "created by orca_2mkl") are spherical
// throughout, carry ORCA's primitive normalisation (one factor per l) and
// the opposite sign of the |m| >= 3 functions.  As in critic2, STO
// basis sets, sp shells, ROHF and fractional occupations are rejected.
bool read_molden(const char *path, HostWfn &w, std::string &err) {
  std::ifstream in(path);
  if (!in) {
    err = std::string("cannot open ") + path;
    return false;
  }
  err = std::string("Error reading file: ") + path;
  std::vector<std::string> lines;
  for (std::string l; std::getline(in, l);) {
    if (!l.empty() && l.back() == '\r') l.pop_back();
    lines.push_back(l);
  }
  auto keyword = [&](size_t i) {
    const std::string l = lower_str(lines[i]);
    const size_t a = l.find('['), b = l.find(']');
    return (a == std::string::npos || b == std::string::npos || b < a) ? std::string() : l.substr(a + 1, b - a - 1);
  };
  bool is5d = false, is7f = false, is9g = false, isorca = false, gto = false, sto = false;
  size_t at_line = 0, gto_line = 0, mo_line = 0;
  double ang = 1.0;
  for (size_t i = 0; i < lines.size(); i++) {
    const std::string k = keyword(i);
    if (k.empty()) continue;
    if (k == "title" && i + 1 < lines.size() && lines[i + 1].find("created by orca_2mkl") != std::string::npos)
      isorca = true;
    else if (k == "atoms") {
      at_line = i + 1;
      if (lower_str(lines[i]).find("angs") != std::string::npos) ang = 1.0 / 0.52917720859;
    } else if (k == "gto") gto = true, gto_line = i + 1;
    else if (k == "sto") sto = true;
    else if (k == "mo") mo_line = i + 1;
    else if (k == "5d" || k == "5d7f") is5d = is7f = true;
    else if (k == "5d10f") is5d = true, is7f = false;
    else if (k == "7f") is5d = false, is7f = true;
    else if (k == "9g") is9g = true;
  }
  if (sto) { err = "STO molden files are not supported"; return false; }
  if (!gto) { err = "No [GTO] or [STO] blocks present"; return false; }
  if (!at_line || !mo_line) return false;
  if (isorca) is5d = is7f = is9g = true;
  // atoms: name index Z x y z
  std::vector<double> xyz;
  std::vector<int> zs;
  for (size_t i = at_line; i < lines.size(); i++) {
    if (lines[i].find('[') != std::string::npos || trim(lines[i]).empty()) break;
    std::istringstream ss(lines[i]);
    std::string name;
    long idx, z;
    double v[3];
    std::string t[3];
    if (!(ss >> name >> idx >> z >> t[0] >> t[1] >> t[2])) return false;
    for (int k = 0; k < 3; k++)
      if (!parse_real(t[k], v[k])) return false;
    zs.push_back((int)z);
    for (int k = 0; k < 3; k++) xyz.push_back(v[k] * ang);
  }
  const int nat = (int)zs.size();
  if (nat == 0) { err = "gto found but no atoms"; return false; }
  // GTO: per atom a header line, then shells "label nprim scale" + primitives, blank line ends the atom
  struct Shell {
    int type, atom;
    std::vector<double> a, c;
  };
  std::vector<Shell> sh;
  size_t i = gto_line;
  for (int a = 0; a < nat; a++) {
    while (i < lines.size() && trim(lines[i]).empty()) i++;
    if (i >= lines.size()) return false;
    i++;  // atom header
    while (i < lines.size() && !trim(lines[i]).empty() && lines[i].find('[') == std::string::npos) {
      std::istringstream ss(lines[i]);
      std::string lab;
      long n = 0;
      if (!(ss >> lab >> n) || n <= 0) { err = "error reading gto block"; return false; }
      lab = lower_str(lab);
      int t;
      if (lab == "s") t = 0;
      else if (lab == "p") t = 1;
      else if (lab == "sp") { err = "SP shells are not supported for molden files"; return false; }
      else if (lab == "d") t = is5d ? -2 : 2;
      else if (lab == "f") t = is7f ? -3 : 3;
      else if (lab == "g") t = is9g ? -4 : 4;
      else { err = "shells above g are not supported for molden files"; return false; }
      Shell s{t, a, {}, {}};
      for (long k = 0; k < n; k++) {
        if (++i >= lines.size()) return false;
        std::istringstream ps(lines[i]);
        std::string ta, tc;
        double va, vc;
        if (!(ps >> ta >> tc) || !parse_real(ta, va) || !parse_real(tc, vc)) return false;
        s.a.push_back(va);
        s.c.push_back(vc);
      }
      sh.push_back(s);
      i++;
    }
  }
  auto nsph = [](int t) { return t < 0 ? 2 * (-t) + 1 : (t + 1) * (t + 2) / 2; };
  long nbas = 0;
  for (const Shell &s : sh) nbas += nsph(s.type);
  // MOs: occupied ones; alpha first, then beta
  struct MO {
    bool alpha;
    int occ;
    std::vector<double> c;
  };
  std::vector<MO> mos;
  bool alpha = true;
  for (size_t j = mo_line; j < lines.size(); j++) {
    const std::string l = lower_str(lines[j]);
    if (l.find("molden format") != std::string::npos) break;
    if (l.find('[') != std::string::npos && l.find("[mo]") == std::string::npos && keyword(j) != "") break;
    if (l.find("spin=") != std::string::npos) alpha = l.find("alpha") != std::string::npos;
    if (l.find("occup=") == std::string::npos) continue;
    double o;
    std::string tok = trim(lines[j].substr(l.find("occup=") + 6));
    if (!parse_real(tok.substr(0, tok.find_first_of(" \t")), o)) { err = "error reading mo block"; return false; }
    const long io = std::lround(o);
    if (std::fabs(o - (double)io) > 1e-6) { err = "Fractional occupations are not supported for molden files"; return false; }
    if (io != 0 && io != 1 && io != 2) { err = "wrong integer occupation"; return false; }
    MO m{alpha, (int)io, std::vector<double>(nbas, 0.0)};
    size_t k = j + 1;
    for (; k < lines.size(); k++) {
      std::istringstream ss(lines[k]);
      std::string ti, tv;
      if (!(ss >> ti >> tv)) break;
      char *end = nullptr;
      const long idx = std::strtol(ti.c_str(), &end, 10);
      if (end == ti.c_str() || *end != '\0') break;
      double v;
      if (!parse_real(tv, v) || idx < 1 || idx > nbas) return false;
      m.c[idx - 1] = v;
    }
    j = k - 1;
    if (io > 0) mos.push_back(m);
  }
  int nelec = 0, nalpha = 0;
  bool beta = false, had1 = false;
  for (const MO &m : mos) {
    nelec += m.occ;
    nalpha += m.alpha ? 1 : 0;
    beta = beta || !m.alpha;
    had1 = had1 || m.occ == 1;
  }
  int wfntyp;
  if (beta) wfntyp = C2G_WFN_UHF;
  else if (had1) { err = "ROHF wavefunctions are not supported for molden files"; return false; }
  else wfntyp = C2G_WFN_RHF;
  if (wfntyp == C2G_WFN_RHF && nelec % 2) { err = "odd nelec but closed-shell wavefunction"; return false; }
  const int nmo = wfntyp == C2G_WFN_UHF ? nelec : nelec / 2;
  std::vector<const MO *> ord;
  for (const MO &m : mos)
    if (m.alpha) ord.push_back(&m);
  for (const MO &m : mos)
    if (!m.alpha) ord.push_back(&m);
  if ((int)ord.size() != nmo) { err = "inconsistent number of MOs"; return false; }
  // ORCA's sign convention for |m| >= 3 (f: 6-7, g: 6-9 of the shell)
  std::vector<std::vector<double>> coef(nmo);
  for (int m = 0; m < nmo; m++) coef[m] = ord[m]->c;
  if (isorca) {
    long ns = 0;
    for (const Shell &s : sh) {
      if (s.type == -3 || s.type == -4)
        for (int m = 0; m < nmo; m++)
          for (int k = 5; k < (s.type == -3 ? 7 : 9); k++) coef[m][ns + k] = -coef[m][ns + k];
      ns += nsph(s.type);
    }
  }
  w = HostWfn();
  w.natom = nat;
  w.nmo = nmo;
  w.xyz = xyz;
  w.z = zs;
  std::vector<std::vector<double>> cols;
  long ns = 0;
  for (const Shell &s : sh) {
    const int l = std::abs(s.type), ncar = (l + 1) * (l + 2) / 2, nsp = nsph(s.type);
    const std::vector<int> types = molden_cart_types(l);
    const double *T = l == 2 ? &kSphCar2[0][0] : l == 3 ? &kSphCar3[0][0] : l == 4 ? &kSphCar4Molden[0][0] : nullptr;
    std::vector<double> car((size_t)nmo * ncar, 0.0);
    for (int m = 0; m < nmo; m++)
      for (int c = 0; c < ncar; c++) {
        if (s.type >= 0 || l < 2) {
          car[(size_t)m * ncar + c] = coef[m][ns + c];
        } else {
          double v = 0.0;
          for (int k = 0; k < nsp; k++) v += coef[m][ns + k] * T[(size_t)k * ncar + c];
          car[(size_t)m * ncar + c] = v;
        }
      }
    const int n = (int)s.a.size();
    for (int c = 0; c < ncar; c++) {
      const int ityp = types[c];
      const int *lv = kLi[ityp - 1];
      std::vector<double> cn(n);
      for (int k = 0; k < n; k++) {
        cn[k] = s.c[k] * gnorm_cart(lv, s.a[k]);
        if (isorca) {
          // ORCA normalises every component of a shell like x^l (gnorm_orca)
          const int xl[3] = {l, 0, 0};
          cn[k] /= gnorm_cart(xl, s.a[k]);
        }
      }
      const double norm = aonorm_cart(lv, n, s.a.data(), cn.data());
      for (int k = 0; k < n; k++) {
        w.icenter.push_back(s.atom);
        w.itype.push_back(ityp);
        w.e.push_back(s.a[k]);
        std::vector<double> col(nmo);
        for (int m = 0; m < nmo; m++) col[m] = cn[k] * norm * car[(size_t)m * ncar + c];
        cols.push_back(col);
      }
    }
    ns += nsp;
  }
  w.npri = (int)w.e.size();
  w.cmo.resize((size_t)w.npri * nmo);
  for (int p = 0; p < w.npri; p++) std::copy(cols[p].begin(), cols[p].end(), w.cmo.begin() + (size_t)p * nmo);
  w.occ.assign(nmo, wfntyp == C2G_WFN_UHF ? 1.0 : 2.0);
  w.wfntyp = wfntyp;
  w.nalpha = nalpha;
  err.clear();
  prune_primitives(w);
  complete_struct(w);
  molecular_cell(w);
  return true;
}

}  // namespace c2g
