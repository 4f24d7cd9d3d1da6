// Media and interaction tables: the host preparation the reference does in
// initMediaData (ompMC src/ompmc.c:5450-5487) and its callees.  Every table
// is rebuilt from the same input files with the same arithmetic, operation
// for operation where the order changes the rounding, so the result is
// bit-identical to the reference's globals (checked against dumps of the
// reference itself).  The transport kernels never see this code: the engine
// repacks these FP64 arrays into its device layouts.
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "common.h"

using omc::fail;
using omc::kRM;

namespace {

constexpr int MXGE = OMC_MXGE;
constexpr int MXEKE = OMC_MXEKE;
constexpr int MXRAYFF = OMC_MXRAYFF;
constexpr int RAYCDFSIZE = OMC_RAYCDFSIZE;
constexpr int MXELEMENT = OMC_MXELEMENT;
constexpr int MXE_SPIN = OMC_MXE_SPIN;
constexpr int MXE_SPIN1 = OMC_MXE_SPIN1;
constexpr int MXQ_SPIN = OMC_MXQ_SPIN;
constexpr int MXU_SPIN = OMC_MXU_SPIN;
constexpr int MXL_MS = OMC_MXL_MS;
constexpr int MXQ_MS = OMC_MXQ_MS;
constexpr int MXU_MS = OMC_MXU_MS;
constexpr double XIMAX = 0.5;    // ompmc.h:191
constexpr double ESTEPE = 0.25;  // ompmc.h:192

struct Element {
  double z = 0, wa = 0, pz = 0, rhoz = 0;
};

struct Medium {
  std::vector<Element> el;
  int msge = 0, mge = 0, mseke = 0, mleke = 0, mcmfp = 0, mrange = 0;
};

double *dalloc(size_t n) { return static_cast<double *>(std::calloc(n ? n : 1, sizeof(double))); }
int *ialloc(size_t n) { return static_cast<int *>(std::calloc(n ? n : 1, sizeof(int))); }

// ---------------------------------------------------------------------------
// pegs4 reader (readPegsFile, ompmc.c:5489-5943).  Only the electron data and
// the header values are read; photon data are rebuilt from XCOM.
// ---------------------------------------------------------------------------

// "NAME = VALUE" items of a comma-separated pegs header line.
void header_items(const std::string &line, std::vector<std::pair<std::string, std::string>> &items) {
  items.clear();
  size_t start = 0;
  while (start <= line.size()) {
    size_t comma = line.find(',', start);
    std::string tok = line.substr(start, comma == std::string::npos ? std::string::npos : comma - start);
    size_t eq = tok.find('=');
    std::string name = omc::remove_spaces(tok.substr(0, eq));
    std::string value = eq == std::string::npos ? std::string() : tok.substr(eq + 1);
    if (!name.empty()) items.emplace_back(name, value);
    if (comma == std::string::npos) break;
    start = comma + 1;
  }
}

omc_status read_pegs(const std::string &path, omc_tables *t, std::vector<Medium> &media) {
  std::string text;
  if (!omc::read_file(path, text)) return fail(OMC_ERR_IO, "Unable to open file: %s", path.c_str());
  // Line start offsets, so that numeric streams can resume at a line.
  std::vector<size_t> starts;
  starts.push_back(0);
  for (size_t i = 0; i < text.size(); i++)
    if (text[i] == '\n') starts.push_back(i + 1);
  auto line_at = [&](size_t li) -> std::string {
    if (li >= starts.size()) return std::string();
    size_t s = starts[li], e = text.find('\n', s);
    if (e == std::string::npos) e = text.size();
    if (e > s && text[e - 1] == '\r') e--;
    return text.substr(s, e - s);
  };
  int nmed = t->nmed, nfound = 0;
  std::vector<int> found(nmed, 0);
  size_t li = 0, nlines = starts.size();
  std::vector<std::pair<std::string, std::string>> items;
  while (nfound < nmed && li < nlines) {
    std::string line = line_at(li++);
    if (line.compare(0, 8, " MEDIUM=") != 0) continue;
    // Name: up to 24 characters after " MEDIUM=", cut at the first space.
    std::string name = line.substr(8, 24);
    size_t sp = name.find(' ');
    if (sp != std::string::npos) name = name.substr(0, sp);
    int imed = -1;
    for (int i = 0; i < nmed; i++)
      if (name == t->names[i]) {
        imed = i;
        break;
      }
    if (imed < 0) continue;
    Medium md;
    int ne = 0;
    bool ok = true;
    header_items(line_at(li++), items);
    for (auto &kv : items) {
      const char *v = kv.second.c_str();
      if (kv.first == "RHO") ok = ok && std::sscanf(v, "%lf", &t->rho[imed]) == 1;
      else if (kv.first == "NE") ok = ok && std::sscanf(v, "%d", &ne) == 1;
    }
    if (!ok || ne < 1) continue;
    for (int m = 0; m < ne && ok; m++) {
      Element e;
      header_items(line_at(li++), items);
      for (auto &kv : items) {
        const char *v = kv.second.c_str();
        if (kv.first == "Z") ok = ok && std::sscanf(v, "%lf", &e.z) == 1;
        else if (kv.first == "A") ok = ok && std::sscanf(v, "%lf", &e.wa) == 1;
        else if (kv.first == "PZ") ok = ok && std::sscanf(v, "%lf", &e.pz) == 1;
        else if (kv.first == "RHOZ") ok = ok && std::sscanf(v, "%lf", &e.rhoz) == 1;
      }
      md.el.push_back(e);
    }
    if (!ok) continue;
    if (std::sscanf(line_at(li++).c_str(), "%lf %lf %lf %lf %lf", &t->rlc[imed], &t->ae[imed], &t->ap[imed],
                    &t->ue[imed], &t->up[imed]) != 5)
      continue;
    t->te[imed] = t->ae[imed] - kRM;
    t->thmoll[imed] = (t->te[imed]) * 2 + kRM;
    int meke = 0;
    if (std::sscanf(line_at(li++).c_str(), "%d %d %d %d %d %d %d", &md.msge, &md.mge, &md.mseke, &meke,
                    &md.mleke, &md.mcmfp, &md.mrange) != 7)
      continue;
    if (meke > MXEKE || meke < 2) continue;
    // Six lines of bremsstrahlung parameters, then a checked line of five.
    li += 6;
    double del[5];
    if (std::sscanf(line_at(li++).c_str(), "%lf %lf %lf %lf %lf", &del[0], &del[1], &del[2], &del[3], &del[4]) != 5)
      continue;
    if (li >= nlines) continue;
    // From here a free-format number stream.
    omc::NumberStream ns(text.c_str() + starts[li]);
    double dl6, alphi1, alphi2, bpar1, bpar2, delpos1, delpos2, xr0, teff0;
    double blcc, xcc, eke0, eke1;
    ok = ns.next(dl6) && ns.next(t->pegs_delcm[imed]) && ns.next(alphi1) && ns.next(alphi2) && ns.next(bpar1) &&
         ns.next(bpar2) && ns.next(delpos1) && ns.next(delpos2) && ns.next(xr0) && ns.next(teff0) &&
         ns.next(blcc) && ns.next(xcc) && ns.next(eke0) && ns.next(eke1);
    if (!ok) return fail(OMC_ERR_FORMAT, "%s: truncated electron header for %s", path.c_str(), name.c_str());
    t->blcc[imed] = blcc;
    t->xcc[imed] = xcc;
    t->eke0[imed] = eke0;
    t->eke1[imed] = eke1;
    double *cols[16] = {t->esig0, t->esig1, t->psig0, t->psig1, t->ededx0, t->ededx1, t->pdedx0, t->pdedx1,
                        t->ebr10, t->ebr11, t->pbr10, t->pbr11, t->pbr20, t->pbr21, t->tmxs0, t->tmxs1};
    for (int k = 0; k < meke && ok; k++)
      for (int c = 0; c < 16 && ok; c++) ok = ns.next(cols[c][imed * MXEKE + k]);
    if (!ok) return fail(OMC_ERR_FORMAT, "%s: truncated electron tables for %s", path.c_str(), name.c_str());
    // Resume line scanning after the last number read.
    size_t off = static_cast<size_t>(ns.pos() - text.c_str());
    while (li < nlines && starts[li] <= off) li++;
    // Length unit: the reference converts radiation lengths to cm.
    double dfacti = 1.0 / (t->rlc[imed]);
    t->blcc[imed] *= dfacti;
    for (int k = 0; k < meke; k++) {
      int i = imed * MXEKE + k;
      t->esig0[i] *= dfacti;
      t->psig0[i] *= dfacti;
      t->ededx0[i] *= dfacti;
      t->pdedx0[i] *= dfacti;
      t->pdedx1[i] *= dfacti;
      t->esig1[i] *= dfacti;
      t->psig1[i] *= dfacti;
      t->ededx1[i] *= dfacti;
    }
    t->xcc[imed] *= std::sqrt(dfacti);
    t->ne[imed] = ne;
    t->meke[imed] = meke;
    media[imed] = md;
    found[imed] = 1;
    nfound++;
  }
  if (nfound < nmed) {
    std::string missing;
    for (int i = 0; i < nmed; i++)
      if (!found[i]) missing += std::string(" ") + t->names[i];
    return fail(OMC_ERR_MEDIA,
                "The following media were not found or could not be read from pegs file %s:%s", path.c_str(),
                missing.c_str());
  }
  for (int i = 0; i < nmed; i++)
    for (const Element &e : media[i].el)
      if (e.z < 1 || e.z > MXELEMENT)
        return fail(OMC_ERR_MEDIA, "medium %s holds Z=%g; the data files cover Z=1..%d", t->names[i], e.z,
                    MXELEMENT);
  return OMC_OK;
}

// ---------------------------------------------------------------------------
// Photon cross sections (initPhotonData, ompmc.c:216-665).
// ---------------------------------------------------------------------------
struct XsecSet {
  std::vector<std::vector<double>> le, ls;  // log energy, log cross section
};

omc_status read_xsec(const std::string &file, XsecSet &x) {
  std::string text;
  if (!omc::read_file(file, text)) return fail(OMC_ERR_IO, "Unable to open file: %s", file.c_str());
  omc::NumberStream ns(text.c_str());
  x.le.assign(MXELEMENT, {});
  x.ls.assign(MXELEMENT, {});
  for (int i = 0; i < MXELEMENT; i++) {
    int n = 0;
    if (!ns.next_int(n) || n < 1) return fail(OMC_ERR_FORMAT, "Could not read the data file %s", file.c_str());
    x.le[i].resize(n);
    x.ls[i].resize(n);
    for (int j = 0; j < n; j++)
      if (!ns.next(x.le[i][j]) || !ns.next(x.ls[i][j]))
        return fail(OMC_ERR_FORMAT, "Could not read the data file %s", file.c_str());
  }
  return OMC_OK;
}

// Medium cross section on the MXGE log-energy grid, summed over elements in
// order of increasing Z (get_data, ompmc.c:347-449).  kind 0: as tabulated;
// kind 1 (pair) / 2 (triplet): threshold 2m / 4m with the (1-eth/E)^3
// extrapolation of the reference.
std::vector<double> medium_xsec(int kind, const XsecSet &x, const std::vector<double> &z_sorted,
                                const std::vector<double> &pz_sorted, double ge0, double ge1) {
  std::vector<double> res(MXGE, 0.0);
  for (size_t i = 0; i < z_sorted.size(); i++) {
    int z = static_cast<int>(z_sorted[i] + 0.5) - 1;
    const std::vector<double> &d0 = x.le[z], &d1 = x.ls[z];
    int n = static_cast<int>(d0.size());
    double eth = 0.0;
    std::vector<double> le, ls;
    if (kind == 0) {
      le = d0;
      ls = d1;
    } else {
      le.assign(n + 1, 0.0);
      ls.assign(n + 1, 0.0);
      for (int j = 0; j < n; j++) {
        le[j + 1] = d0[j];
        ls[j + 1] = d1[j];
      }
      eth = (kind == 1) ? 2.0 * kRM : 4.0 * kRM;
      n++;
      for (int j = 1; j < n; j++) ls[j] -= 3.0 * std::log(1.0 - eth / std::exp(le[j]));
      le[0] = std::log(eth);
      ls[0] = ls[1];
    }
    for (int j = 0; j < MXGE; j++) {
      double gle = (static_cast<double>(j + 1) - ge0) / ge1;
      double e = std::exp(gle);
      double sig = 0.0;
      if (gle < le[0] || gle >= le[n - 1]) {
        if (kind != 0) sig = (gle < le[0]) ? 0.0 : std::exp(ls[n - 1]);
      } else {
        int k = 0;
        while (k < n - 1 && !(gle >= le[k] && gle < le[k + 1])) k++;
        if (k >= n - 1) k = n - 2;  // unreachable for sorted data
        double p = (gle - le[k]) / (le[k + 1] - le[k]);
        sig = std::exp(p * ls[k + 1] + (1.0 - p) * ls[k]);
      }
      if (kind != 0 && e > eth) sig *= (1.0 - eth / e) * (1.0 - eth / e) * (1.0 - eth / e);
      res[j] += pz_sorted[i] * sig;
    }
  }
  return res;
}

// Klein-Nishina total cross section per electron (kn_sigma0, ompmc.c:451).
double kn_sigma0(double e) {
  const double con = 0.1274783851;
  double ko = e / kRM;
  if (ko < 0.01) return 8.0 * con / 3.0 * (1.0 - ko * (2.0 - ko * (5.2 - 13.3 * ko))) / kRM;
  double c1 = 1.0 / (ko * ko);
  double c2 = 1.0 - 2.0 * (1.0 + ko) * c1;
  double c3 = (1.0 + 2.0 * ko) * c1;
  double eps2 = 1.0;
  double eps1 = 1.0 / (1.0 + 2.0 * ko);
  return (c1 * (1.0 / eps1 - 1.0 / eps2) + c2 * std::log(eps2 / eps1) + eps2 * (c3 + 0.5 * eps2) -
          eps1 * (c3 + 0.5 * eps1)) /
         e * con;
}

// Piecewise-linear coefficients on the uniform log grid: value_j at
// gle_j = (j+1-ge0)/ge1 becomes (c1, c0) with c1*gle + c0, interval j-1
// holding the segment ending at j; the last interval repeats the slope.
void pwl_coeffs(const std::vector<double> &val, const std::vector<double> &gle, double ge1, double *c0, double *c1,
                int n) {
  for (int j = 1; j < n; j++) {
    c1[j - 1] = (val[j] - val[j - 1]) * ge1;
    c0[j - 1] = val[j] - c1[j - 1] * gle[j];
  }
  c1[n - 1] = c1[n - 2];
  c0[n - 1] = val[n - 1] - c1[n - 1] * gle[n - 1];
}

omc_status build_photon(omc_tables *t, const std::vector<Medium> &media, const std::string &folder) {
  XsecSet photo, rayl, pair, trip;
  omc_status s;
  if ((s = read_xsec(folder + "xcom_photo.data", photo)) != OMC_OK) return s;
  if ((s = read_xsec(folder + "xcom_rayleigh.data", rayl)) != OMC_OK) return s;
  if ((s = read_xsec(folder + "xcom_pair.data", pair)) != OMC_OK) return s;
  if ((s = read_xsec(folder + "xcom_triplet.data", trip)) != OMC_OK) return s;
  for (int i = 0; i < t->nmed; i++) {
    const std::vector<Element> &el = media[i].el;
    t->ge1[i] = static_cast<double>(MXGE - 1) / std::log(t->up[i] / t->ap[i]);
    t->ge0[i] = 1.0 - t->ge1[i] * std::log(t->ap[i]);
    double sumA = 0.0, sumZ = 0.0;
    for (const Element &e : el) {
      sumA += e.pz * e.wa;
      sumZ += e.pz * e.z;
    }
    double con2 = t->rho[i] / (sumA * 1.6605655);
    // Elements ordered by increasing Z (heap_sort, ompmc.c:280).
    std::vector<int> order(el.size());
    for (size_t j = 0; j < el.size(); j++) order[j] = static_cast<int>(j);
    for (size_t a = 1; a < order.size(); a++)
      for (size_t b = a; b > 0 && el[order[b]].z < el[order[b - 1]].z; b--) std::swap(order[b], order[b - 1]);
    std::vector<double> z_sorted(el.size()), pz_sorted(el.size());
    for (size_t j = 0; j < el.size(); j++) {
      z_sorted[j] = el[order[j]].z;
      pz_sorted[j] = el[order[j]].pz;
    }
    double ge0 = t->ge0[i], ge1 = t->ge1[i];
    std::vector<double> sp = medium_xsec(0, photo, z_sorted, pz_sorted, ge0, ge1);
    std::vector<double> sr = medium_xsec(0, rayl, z_sorted, pz_sorted, ge0, ge1);
    std::vector<double> spair = medium_xsec(1, pair, z_sorted, pz_sorted, ge0, ge1);
    std::vector<double> strip = medium_xsec(2, trip, z_sorted, pz_sorted, ge0, ge1);
    std::vector<double> gle(MXGE), gmfp(MXGE), gbr1(MXGE), gbr2(MXGE), cohe(MXGE);
    for (int j = 0; j < MXGE; j++) {
      gle[j] = (static_cast<double>(j + 1) - ge0) / ge1;
      double e = std::exp(gle[j]);
      double sig_kn = sumZ * kn_sigma0(e);
      double sig_p = spair[j] + strip[j];
      double sigma = sig_kn + sig_p + sp[j];
      gmfp[j] = 1.0 / (sigma * con2);
      gbr1[j] = sig_p / sigma;
      gbr2[j] = gbr1[j] + sig_kn / sigma;
      cohe[j] = sigma / (sr[j] + sigma);
    }
    size_t o = static_cast<size_t>(i) * MXGE;
    pwl_coeffs(gmfp, gle, ge1, t->gmfp0 + o, t->gmfp1 + o, MXGE);
    pwl_coeffs(gbr1, gle, ge1, t->gbr10 + o, t->gbr11 + o, MXGE);
    pwl_coeffs(gbr2, gle, ge1, t->gbr20 + o, t->gbr21 + o, MXGE);
    pwl_coeffs(cohe, gle, ge1, t->cohe0 + o, t->cohe1 + o, MXGE);
  }
  return OMC_OK;
}

// ---------------------------------------------------------------------------
// Rayleigh form-factor sampling tables (initRayleighData, ompmc.c:820-1007).
// ---------------------------------------------------------------------------
omc_status build_rayleigh(omc_tables *t, const std::vector<Medium> &media, const std::string &pgs4form) {
  std::string text;
  if (!omc::read_file(pgs4form, text)) return fail(OMC_ERR_IO, "Unable to open file: %s", pgs4form.c_str());
  omc::NumberStream ns(text.c_str());
  std::vector<double> xval(MXRAYFF);
  std::vector<std::vector<double>> aff(MXELEMENT, std::vector<double>(MXRAYFF));
  for (int i = 0; i < MXRAYFF; i++)
    if (!ns.next(xval[i])) return fail(OMC_ERR_FORMAT, "Could not read atomic form factors file %s", pgs4form.c_str());
  for (int i = 0; i < MXELEMENT; i++)
    for (int j = 0; j < MXRAYFF; j++)
      if (!ns.next(aff[i][j]))
        return fail(OMC_ERR_FORMAT, "Could not read atomic form factors file %s", pgs4form.c_str());
  std::vector<double> ff(MXRAYFF), pe(MXGE);
  for (int i = 0; i < t->nmed; i++) {
    double *xg = t->xgrid + i * MXRAYFF, *fc = t->fcum + i * MXRAYFF;
    double *ba = t->b_array + i * MXRAYFF, *ca = t->c_array + i * MXRAYFF;
    int *ia = t->i_array + i * RAYCDFSIZE;
    // Independent-atom form factor of the mixture.
    for (int j = 0; j < MXRAYFF; j++) {
      double ffv = 0.0;
      xg[j] = xval[j];
      for (const Element &e : media[i].el) {
        int z = static_cast<int>(e.z) - 1;
        ffv += e.pz * std::pow(aff[z][j], 2);
      }
      ff[j] = std::sqrt(ffv);
    }
    if (xg[0] < 1.0E-6) xg[0] = 0.0001;
    double emin = std::exp((1.0 - t->ge0[i]) / t->ge1[i]);
    double emax = std::exp((MXGE - t->ge0[i]) / t->ge1[i]);
    for (int j = 0; j < MXRAYFF; j++) {  // avoid log(0): +0.0 -> smallest subnormal
      uint64_t bits;
      std::memcpy(&bits, &ff[j], 8);
      if (bits == 0) {
        bits = 1;
        std::memcpy(&ff[j], &bits, 8);
      }
    }
    // Cumulative distribution on the form-factor grid.
    double sum0 = 0.0;
    fc[0] = 0.0;
    for (int j = 0; j < MXRAYFF - 1; j++) {
      double b = std::log(ff[j + 1] / ff[j]) / std::log(xg[j + 1] / xg[j]);
      ba[j] = b;
      double x1 = xg[j], x2 = xg[j + 1];
      double px1 = std::pow(x1, 2.0 * b), px2 = std::pow(x2, 2.0 * b);
      sum0 += std::pow(ff[j], 2) * (std::pow(x2, 2) * px2 - std::pow(x1, 2) * px1) / ((1.0 + b) * px1);
      fc[j + 1] = sum0;
    }
    // Maximum cumulative probability as a function of photon energy.
    double dle = std::log(emax / emin) / (static_cast<double>(MXGE) - 1.0);
    int idx = 1;
    for (int j = 1; j <= MXGE; j++) {
      double e = emin * std::exp(dle * (static_cast<double>(j) - 1.0));
      double xmax = 20.607544 * 2.0 * e / kRM;
      int k = 1;
      while (k <= MXRAYFF - 1 && !(xmax >= xg[k - 1] && xmax < xg[k])) k++;
      idx = k;
      double b = ba[idx - 1], x1 = xg[idx - 1], x2 = xmax;
      double px1 = std::pow(x1, 2.0 * b), px2 = std::pow(x2, 2.0 * b);
      pe[j - 1] = fc[idx - 1] + std::pow(ff[idx - 1], 2) * (std::pow(x2, 2) * px2 - std::pow(x1, 2) * px1) /
                                    ((1.0 + b) * px1);
    }
    ia[RAYCDFSIZE - 1] = idx;
    // Normalise so that pe(emax) = 1, with pe slightly enlarged so that
    // fcum(xmax) is never underestimated by interpolation.
    double anorm = 1.0 / std::sqrt(pe[MXGE - 1]);
    double anorm1 = 1.005 / pe[MXGE - 1];
    double anorm2 = 1.0 / pe[MXGE - 1];
    for (int j = 0; j < MXGE; j++) {
      pe[j] *= anorm1;
      if (pe[j] > 1.0) pe[j] = 1.0;
    }
    for (int j = 0; j < MXRAYFF; j++) {
      ff[j] *= anorm;
      fc[j] *= anorm2;
      ca[j] = (1.0 + ba[j]) / std::pow(xg[j] * ff[j], 2);
    }
    // Uniform cumulative bins -> first form-factor interval of each bin.
    double dw = 1.0 / (static_cast<double>(RAYCDFSIZE) - 1.0);
    double xold = xg[0];
    int ibin = 1;
    double b = ba[0];
    double px1 = std::pow(xg[0], 2.0 * b);
    ia[0] = 1;
    for (int j = 2; j <= RAYCDFSIZE - 1; j++) {
      double w = dw;
      for (int guard = 0;; guard++) {
        if (ibin >= MXRAYFF || guard > 4 * MXRAYFF)
          return fail(OMC_ERR_FORMAT, "Rayleigh CDF construction failed for medium %s", t->names[i]);
        double x1 = xold, x2 = xg[ibin];
        double tt = std::pow(x1, 2) * std::pow(x1, 2.0 * b);
        double px2 = std::pow(x2, 2.0 * b);
        double aux = std::pow(ff[ibin - 1], 2) * (std::pow(x2, 2) * px2 - tt) / ((1.0 + b) * px1);
        if (aux > w) {
          xold = std::exp(std::log(tt + w * (1.0 + b) * px1 / std::pow(ff[ibin - 1], 2)) / (2.0 + 2.0 * b));
          ia[j - 1] = ibin;
          break;
        }
        w -= aux;
        xold = x2;
        ibin++;
        b = ba[ibin - 1];
        px1 = std::pow(xold, 2.0 * b);
      }
    }
    for (int j = 0; j < MXRAYFF; j++) ba[j] = 0.5 / (1.0 + ba[j]);
    double *p0 = t->pmax0 + i * MXGE, *p1 = t->pmax1 + i * MXGE;
    for (int j = 0; j < MXGE - 1; j++) {
      double gle = ((j + 1) - t->ge0[i]) / t->ge1[i];
      p1[j] = (pe[j + 1] - pe[j]) * t->ge1[i];
      p0[j] = pe[j] - p1[j] * gle;
    }
    p0[MXGE - 1] = p0[MXGE - 2];
    p1[MXGE - 1] = p1[MXGE - 2];
  }
  return OMC_OK;
}

// ---------------------------------------------------------------------------
// Pair / bremsstrahlung screening parameters (initPairData, ompmc.c:1148-1318).
// ---------------------------------------------------------------------------
double coulomb_correction(double zi) {  // fcoulc, ompmc.c:1148
  double a = 0.00729735255664 * zi;
  double fc = 1 + std::pow(a, 2);
  fc = 1.0 / fc;
  fc = fc + 0.20206 - 0.0369 * std::pow(a, 2);
  fc = fc + 0.0083 * std::pow(a, 4);
  fc = fc - 0.002 * std::pow(a, 6);
  fc = fc * std::pow(a, 2);
  return fc;
}

double atomic_electron_term(double zi, double fc) {  // xsif, ompmc.c:1165
  if (zi == 4) return 5.924 / (4.710 - fc);
  if (zi == 3) return 5.805 / (4.740 - fc);
  if (zi == 2) return 5.621 / (4.790 - fc);
  if (zi == 1) return 6.144 / (5.310 - fc);
  return std::log(1194.0 * std::pow(zi, -2.0 / 3.0)) / std::log(184.15 * std::pow(zi, -1.0 / 3.0)) - fc;
}

void build_pair(omc_tables *t, const std::vector<Medium> &media) {
  for (int m = 0; m < t->nmed; m++) {
    double Zt = 0.0, Zb = 0.0, Zf = 0.0;
    for (const Element &e : media[m].el) {
      double fc = coulomb_correction(e.z);
      double xi = atomic_electron_term(e.z, fc);
      double aux = e.pz * e.z * (e.z + xi);
      Zt = Zt + aux;
      Zb = Zb - aux * std::log(e.z) / 3.0;
      Zf = Zf + aux * fc;
    }
    double Zv = (Zb - Zf) / Zt;
    double Zg = Zb / Zt;
    double fmax1 = 2.0 * (20.863 + 4.0 * Zg) - 2.0 * (20.029 + 4.0 * Zg) / 3.0;
    double fmax2 = 2.0 * (20.863 + 4.0 * Zv) - 2.0 * (20.029 + 4.0 * Zv) / 3.0;
    double *d1 = t->dl1 + 8 * m, *d2 = t->dl2 + 8 * m, *d3 = t->dl3 + 8 * m;
    double *d4 = t->dl4 + 8 * m, *d5 = t->dl5 + 8 * m, *d6 = t->dl6 + 8 * m;
    // Sets 0-3: bremsstrahlung (screening Zg / Coulomb-corrected Zv),
    // normalised by their maxima; sets 4-7: pair production.
    const double zs[2] = {Zg, Zv}, fm[2] = {fmax1, fmax2};
    for (int c = 0; c < 2; c++) {
      int a = 2 * c, b = 2 * c + 1;
      d1[a] = (20.863 + 4.0 * zs[c]) / fm[c];
      d2[a] = -3.242 / fm[c];
      d3[a] = 0.625 / fm[c];
      d4[a] = (21.12 + 4.0 * zs[c]) / fm[c];
      d5[a] = -4.184 / fm[c];
      d6[a] = 0.952;
      d1[b] = (20.029 + 4.0 * zs[c]) / fm[c];
      d2[b] = -1.93 / fm[c];
      d3[b] = -0.086 / fm[c];
      d4[b] = (21.12 + 4.0 * zs[c]) / fm[c];
      d5[b] = -4.184 / fm[c];
      d6[b] = 0.952;
    }
    for (int c = 0; c < 2; c++) {
      int a = 4 + 2 * c, b = 5 + 2 * c;
      d1[a] = (3.0 * (20.863 + 4.0 * zs[c]) - (20.029 + 4.0 * zs[c]));
      d2[a] = (3.0 * (-3.242) - (-1.930));
      d3[a] = (3.0 * (0.625) - (-0.086));
      d4[a] = (2.0 * 21.12 + 8.0 * zs[c]);
      d5[a] = (2.0 * (-4.184));
      d6[a] = 0.952;
      d1[b] = (3.0 * (20.863 + 4.0 * zs[c]) + (20.029 + 4.0 * zs[c]));
      d2[b] = (3.0 * (-3.242) + (-1.930));
      d3[b] = (3.0 * 0.625 + (-0.086));
      d4[b] = (4.0 * 21.12 + 16.0 * zs[c]);
      d5[b] = (4.0 * (-4.184));
      d6[b] = 0.952;
    }
    t->bpar1[m] = d1[6] / (3.0 * d1[7] + d1[6]);
    t->bpar0[m] = 12.0 * d1[7] / (3.0 * d1[7] + d1[6]);
    // Composite angular factor ((1/111) Zeff^(1/3))^2.
    double zbr = 0.0, pznorm = 0.0;
    for (const Element &e : media[m].el) {
      zbr += static_cast<double>(e.pz) * (e.z) * ((e.z) + 1.0);
      pznorm += e.pz;
    }
    t->zbrang[m] = (8.116224E-05) * std::pow(zbr / pznorm, 1.0 / 3.0);
    t->delcm[m] = t->pegs_delcm[m];
  }
}

// ---------------------------------------------------------------------------
// Spline through (x, f) (setSpline / spline, ompmc.c:3016-3095).
// ---------------------------------------------------------------------------
void spline_setup(const double *x, const double *f, double *a, double *b, double *c, double *d, int n) {
  int m1 = 2, m2 = n - 1;
  double s = 0, r;
  for (int m = 1; m <= m2; m++) {
    d[m - 1] = x[m] - x[m - 1];
    r = (f[m] - f[m - 1]) / d[m - 1];
    c[m - 1] = r - s;
    s = r;
  }
  s = 0;
  r = 0;
  c[0] = 0;
  c[n - 1] = 0;
  for (int m = m1; m <= m2; m++) {
    c[m - 1] = c[m - 1] + r * c[m - 2];
    b[m - 1] = 2 * (x[m - 2] - x[m]) - r * s;
    s = d[m - 1];
    r = s / b[m - 1];
  }
  int mr = m2;
  for (int m = m1; m <= m2; m++) {
    c[mr - 1] = (d[mr - 1] * c[mr] - c[mr - 1]) / b[mr - 1];
    mr = mr - 1;
  }
  for (int m = 1; m <= m2; m++) {
    s = d[m - 1];
    r = c[m] - c[m - 1];
    d[m - 1] = r / s;
    c[m - 1] = 3 * c[m - 1];
    b[m - 1] = (f[m] - f[m - 1]) / s - (c[m - 1] + r) * s;
    a[m - 1] = f[m - 1];
  }
}

double spline_eval(double s, const double *x, const double *a, const double *b, const double *c, const double *d,
                   int n) {
  int dir, mlo, mup, m;
  if (x[0] > x[n - 1]) {
    dir = 1;
    mlo = n;
    mup = 0;
  } else {
    dir = 0;
    mlo = 0;
    mup = n;
  }
  if (s >= x[mup + dir - 1]) {
    m = mup + 2 * dir - 1;
  } else if (s <= x[mlo - dir]) {
    m = mlo - 2 * dir + 1;
  } else {
    int ml = mlo, mu = mup;
    while (std::abs(mu - ml) > 1) {
      int mav = (ml + mu) / 2;
      if (s < x[mav - 1]) mu = mav;
      else ml = mav;
    }
    m = mu + dir - 1;
  }
  double q = s - x[m - 1];
  return a[m - 1] + q * (b[m - 1] + q * (c[m - 1] + q * d[m - 1]));
}

// ---------------------------------------------------------------------------
// Multiple scattering: msnew q-surface (readRutherfordMscat, ompmc.c:3201),
// spin corrections (initSpinData, :2376) and the range / maximum step tables
// (initMscatData, :3282-3511).
// ---------------------------------------------------------------------------
omc_status read_msnew(omc_tables *t, const std::string &file) {
  std::string text;
  if (!omc::read_file(file, text)) return fail(OMC_ERR_IO, "Unable to open file: %s", file.c_str());
  omc::NumberStream ns(text.c_str());
  for (int i = 0; i <= MXL_MS; i++)
    for (int j = 0; j <= MXQ_MS; j++) {
      int base = i * (MXQ_MS + 1) * (MXU_MS + 1) + j * (MXU_MS + 1);
      bool ok = true;
      for (int k = 0; k <= MXU_MS; k++) ok = ok && ns.next(t->ums[base + k]);
      for (int k = 0; k <= MXU_MS; k++) ok = ok && ns.next(t->fms[base + k]);
      for (int k = 0; k < MXU_MS; k++) ok = ok && ns.next(t->wms[base + k]);
      for (int k = 0; k < MXU_MS; k++) ok = ok && ns.next_int(t->ims[base + k]);
      if (!ok) return fail(OMC_ERR_FORMAT, "Could not read multiple-scattering data file %s", file.c_str());
      for (int k = 0; k < MXU_MS; k++) {
        t->fms[base + k] = t->fms[base + k + 1] / t->fms[base + k] - 1.0;
        t->ims[base + k] = t->ims[base + k] - 1;
      }
      t->fms[base + MXU_MS] = t->fms[base + MXU_MS - 1];
    }
  double llammin = std::log(1.0), llammax = std::log(1.0E5);
  double dllamb = (llammax - llammin) / MXL_MS;
  t->dllambi = 1.0 / dllamb;
  double dqms = 0.5 / MXQ_MS;
  t->dqmsi = 1.0 / dqms;
  return OMC_OK;
}

omc_status build_spin(omc_tables *t, const std::vector<Medium> &media, const std::string &file) {
  std::string raw;
  if (!omc::read_file(file, raw)) return fail(OMC_ERR_IO, "Unable to open file: %s", file.c_str());
  const size_t rec_bytes = 276 * 4;
  if (raw.size() < rec_bytes) return fail(OMC_ERR_FORMAT, "spin data file %s is truncated", file.c_str());
  auto f32 = [&](size_t byte) {
    float v;
    std::memcpy(&v, raw.data() + byte, 4);
    return v;
  };
  auto i16 = [&](size_t byte) {
    int16_t v;
    std::memcpy(&v, raw.data() + byte, 2);
    return v;
  };
  // Header: 32-byte version, 4-byte endianness tag, four float32.
  float espin_min = f32(36), espin_max = f32(40), b2spin_min = f32(44), b2spin_max = f32(48);
  t->b2spin_min = static_cast<double>(b2spin_min);
  const int nener = MXE_SPIN;
  // Energy grid (keV): log-spaced below espin_max, beta^2-spaced above.  The
  // float/float divisions are as in the reference (single precision).
  double earray[MXE_SPIN1 + 2];
  double dloge = std::log(static_cast<double>(espin_max / espin_min)) / static_cast<double>(nener);
  double eloge = std::log(static_cast<double>(espin_min));
  earray[0] = espin_min;
  for (int i = 1; i <= nener; i++) {
    eloge += dloge;
    earray[i] = std::exp(eloge);
  }
  double dbeta2 = static_cast<float>((b2spin_max - b2spin_min) / static_cast<float>(nener));
  double beta2 = b2spin_min;
  earray[nener + 1] = espin_max;
  for (int i = nener + 2; i <= 2 * nener + 1; i++) {
    beta2 += dbeta2;
    earray[i] = (beta2 < 0.999) ? kRM * 1000.0 * (1.0 / std::sqrt(1.0 - beta2) - 1) : 50585.1;
  }
  espin_min = static_cast<float>(espin_min / 1000.0);
  espin_max = static_cast<float>(espin_max / 1000.0);
  double dlener = std::log(static_cast<double>(espin_max / espin_min)) / MXE_SPIN;
  t->dleneri = 1.0 / dlener;
  t->espml = std::log(static_cast<double>(espin_min));
  dbeta2 = static_cast<float>((b2spin_max - b2spin_min) / static_cast<float>(MXE_SPIN));
  t->dbeta2i = 1.0 / dbeta2;
  double dqq1 = 0.5 / MXQ_SPIN;
  t->dqq1i = 1.0 / dqq1;

  const int NE1 = MXE_SPIN1 + 1, NQ = MXQ_SPIN + 1, NU = MXU_SPIN + 1;
  const double fsc_tf = 137.03604 * 0.88534138;
  for (int imed = 0; imed < t->nmed; imed++) {
    double eta_a[2][MXE_SPIN1 + 1] = {}, c_a[2][MXE_SPIN1 + 1] = {}, g_a[2][MXE_SPIN1 + 1] = {};
    double *rej = t->spin_rej + static_cast<size_t>(imed) * 2 * NE1 * NQ * NU;
    double sum_Z2 = 0.0, sum_A = 0.0, sum_pz = 0.0, sum_Z = 0.0;
    for (const Element &el : media[imed].el) {
      double z = el.z;
      int iz = static_cast<int>(z + 0.5);
      double pz = el.pz;
      double tmp = z * (z + 1.0) * pz;
      sum_Z2 += tmp;
      sum_Z += pz * z;
      sum_A += pz * el.wa;
      sum_pz += pz;
      double z23 = std::pow(z, 2.0 / 3.0);
      for (int iq = 0; iq < 2; iq++)
        for (int i = 0; i <= MXE_SPIN1; i++) {
          size_t irec = 1 + static_cast<size_t>(iz - 1) * 4 * (nener + 1) + 2 * iq * (nener + 1) + i + 1;
          size_t off = rec_bytes * (irec - 1);
          if (off + rec_bytes > raw.size())
            return fail(OMC_ERR_FORMAT, "spin data file %s has no record for Z=%d", file.c_str(), iz);
          double dum1 = f32(off), dum2 = f32(off + 4), dum3 = f32(off + 8), aux_o = f32(off + 12);
          double fmax[MXQ_SPIN + 1];
          for (int q = 0; q <= MXQ_SPIN; q++) fmax[q] = f32(off + 16 + 4 * q);
          eta_a[iq][i] += tmp * std::log(z23 * aux_o);
          double tau = earray[i] / (1000.0 * kRM);
          double eta = z23 / (fsc_tf * fsc_tf) * aux_o / 4 / tau / (tau + 2);
          c_a[iq][i] += tmp * (std::log(1.0 + 1.0 / eta) - 1.0 / (1.0 + eta)) * dum1 * dum3;
          g_a[iq][i] += tmp * dum2;
          double *r = rej + (static_cast<size_t>(iq) * NE1 + i) * NQ * NU;
          for (int j = 0; j <= MXQ_SPIN; j++)
            for (int k = 0; k <= MXU_SPIN; k++) {
              int ii2 = i16(off + 80 + 2 * (static_cast<size_t>(NU) * j + k));
              if (ii2 < 0) ii2 += 65536;
              double d = ii2;
              d = d * fmax[j] / 65535;
              r[j * NU + k] += tmp * d;
            }
        }
    }
    // Rejection function scaled to a maximum of one per (iq, i, j).
    for (int row = 0; row < 2 * NE1 * NQ; row++) {
      double *r = rej + static_cast<size_t>(row) * NU, flmax = 0.0;
      for (int k = 0; k < NU; k++)
        if (flmax < r[k]) flmax = r[k];
      for (int k = 0; k < NU; k++) r[k] = r[k] / flmax;
    }
    for (int i = 0; i <= MXE_SPIN1; i++) {
      double tau = (earray[i] / kRM) * 0.001;
      for (int iq = 0; iq < 2; iq++) {
        double aux_o = std::exp(eta_a[iq][i] / sum_Z2) / (std::pow(fsc_tf, 2.0));
        eta_a[iq][i] = 0.26112447 * aux_o * (t->blcc[imed]) / (t->xcc[imed]);
        double eta = aux_o / 4.0 / tau / (tau + 2);
        double lg = std::log(1.0 + 1.0 / eta);
        double gamma = 3.0 * (1.0 + eta) * (lg * (1.0 + 2.0 * eta) - 2.0) / (lg * (1.0 + eta) - 1.0);
        g_a[iq][i] = g_a[iq][i] / sum_Z2 / gamma;
        c_a[iq][i] = c_a[iq][i] / sum_Z2 / (std::log(1.0 + 1.0 / eta) - 1.0 / (1.0 + eta));
      }
    }
    // Screening correction etap on the electron energy grid.
    double eke0 = t->eke0[imed], eke1 = t->eke1[imed];
    int neke = t->meke[imed];
    size_t o = static_cast<size_t>(imed) * MXEKE;
    auto eta_at = [&](double eil, double e, double &se, double &sp, bool first) {
      if (e <= espin_min) {
        se = eta_a[0][0];
        sp = eta_a[1][0];
        return;
      }
      double aae;
      int je;
      if (e <= espin_max) {
        aae = (eil - t->espml) * t->dleneri;
        je = static_cast<int>(aae);
        aae = aae - je;
      } else {
        double tau = e / kRM;
        // The reference writes the first grid point with pow() and the rest
        // with a product (ompmc.c:2688, 2716).
        double b2 = first ? tau * (tau + 2.0) / std::pow(tau + 1.0, 2.0)
                          : tau * (tau + 2.0) / ((tau + 1.0) * (tau + 1.0));
        aae = (b2 - t->b2spin_min) * t->dbeta2i;
        je = static_cast<int>(aae);
        aae = aae - je;
        je = je + MXE_SPIN + 1;
      }
      se = (1.0 - aae) * eta_a[0][je] + aae * eta_a[0][je + 1];
      sp = (1.0 - aae) * eta_a[1][je] + aae * eta_a[1][je + 1];
    };
    double eil = (1.0 - eke0) / eke1, si1e, si1p, si2e, si2p;
    eta_at(eil, std::exp(eil), si1e, si1p, true);
    for (int i = 1; i < neke; i++) {
      eil = (i + 1.0 - eke0) / eke1;
      eta_at(eil, std::exp(eil), si2e, si2p, false);
      t->etae_ms1[o + i - 1] = (si2e - si1e) * eke1;
      t->etae_ms0[o + i - 1] = (si2e - t->etae_ms1[o + i - 1] * eil);
      t->etap_ms1[o + i - 1] = (si2p - si1p) * eke1;
      t->etap_ms0[o + i - 1] = (si2p - t->etap_ms1[o + i - 1] * eil);
      si1e = si2e;
      si1p = si2p;
    }
    t->etae_ms1[o + neke - 1] = t->etae_ms1[o + neke - 2];
    t->etae_ms0[o + neke - 1] = t->etae_ms0[o + neke - 2];
    t->etap_ms1[o + neke - 1] = t->etap_ms1[o + neke - 2];
    t->etap_ms0[o + neke - 1] = t->etap_ms0[o + neke - 2];
    // First and second moment corrections: a spline in log energy (MeV)
    // through the 31 distinct grid points plus (max(ue, 1e5), 1).
    const int ndata = MXE_SPIN1 + 1;
    double elarray[MXE_SPIN1 + 1], farray[MXE_SPIN1 + 1];
    double af[MXE_SPIN1 + 1], bf[MXE_SPIN1 + 1], cf[MXE_SPIN1 + 1], df[MXE_SPIN1 + 1];
    for (int i = 0; i <= MXE_SPIN; i++) elarray[i] = std::log(earray[i] / 1000.0);
    for (int i = MXE_SPIN + 1; i <= MXE_SPIN1 - 1; i++) elarray[i] = std::log(earray[i + 1] / 1000.0);
    elarray[ndata - 1] = (t->ue[imed] > 1.0E5) ? std::log(t->ue[imed]) : std::log(1.0E5);
    auto moment_table = [&](const double *src, double *c0, double *c1, bool last_from_slope) {
      for (int i = 0; i <= MXE_SPIN; i++) farray[i] = src[i];
      for (int i = MXE_SPIN + 1; i <= MXE_SPIN1 - 1; i++) farray[i] = src[i + 1];
      farray[ndata - 1] = 1.0;
      spline_setup(elarray, farray, af, bf, cf, df, ndata);
      double x = (1.0 - eke0) / eke1;
      double s1 = spline_eval(x, elarray, af, bf, cf, df, ndata);
      for (int i = 1; i <= neke - 1; i++) {
        x = (i + 1 - eke0) / eke1;
        double s2 = spline_eval(x, elarray, af, bf, cf, df, ndata);
        c1[o + i - 1] = (s2 - s1) * eke1;
        c0[o + i - 1] = s2 - c1[o + i - 1] * x;
        s1 = s2;
      }
      c1[o + neke - 1] = c1[o + neke - 2];
      // The reference copies the SLOPE into the last intercept of q1ce
      // (ompmc.c:2784-2785); kept for identical tables.
      c0[o + neke - 1] = last_from_slope ? c1[o + neke - 2] : c0[o + neke - 2];
    };
    moment_table(c_a[0], t->q1ce_ms0, t->q1ce_ms1, true);
    moment_table(c_a[1], t->q1cp_ms0, t->q1cp_ms1, false);
    moment_table(g_a[0], t->q2ce_ms0, t->q2ce_ms1, false);
    moment_table(g_a[1], t->q2cp_ms0, t->q2cp_ms1, false);
    // Scattering power already taken by discrete Moller events.
    double tauc = t->te[imed] / kRM;
    si1e = 1.0;
    for (int i = 1; i <= neke - 1; i++) {
      eil = (static_cast<double>(i + 1) - eke0) / eke1;
      double e = std::exp(eil);
      int leil = i;
      double tau = e / kRM;
      si2e = 1.0;
      if (tau > 2.0 * tauc) {
        double sig = t->esig1[o + leil] * eil + t->esig0[o + leil];
        double dedx = t->ededx1[o + leil] * eil + t->ededx0[o + leil];
        sig /= dedx;
        if (sig > 1.0E-6) {
          double etap = t->etae_ms1[o + leil] * eil + t->etae_ms0[o + leil];
          double eta = 0.25 * etap * (t->xcc[imed]) / (t->blcc[imed]) / tau / (tau + 2);
          double g_r = (1.0 + 2.0 * eta) * std::log(1.0 + 1.0 / eta) - 2.0;
          double p = (tau + 2.0) / (tau + 1.0);
          double tp1sq = (tau + 1.0) * (tau + 1.0);
          double g_m = std::log(0.5 * tau / tauc) +
                       (1.0 + p * p) * std::log(2.0 * (tau - tauc + 2.0) / (tau + 4.0)) -
                       0.25 * (tau + 2.0) * (tau + 2.0 + 2.0 * (2.0 * tau + 1.0) / tp1sq) *
                           std::log((tau + 4.0) * (tau - tauc) / tau / (tau - tauc + 2.0)) +
                       0.5 * (tau - 2.0 * tauc) * (tau + 2.0) * (1.0 / (tau - tauc) - 1.0 / tp1sq);
          g_m = (g_m < g_r) ? g_m / g_r : 1.0;
          si2e = 1.0 - g_m * sum_Z / sum_Z2;
        }
      }
      t->blcce1[o + i - 1] = (si2e - si1e) * eke1;
      t->blcce0[o + i - 1] = si2e - t->blcce1[o + i - 1] * eil;
      si1e = si2e;
    }
    t->blcce1[o + neke - 1] = t->blcce1[o + neke - 2];
    t->blcce0[o + neke - 1] = t->blcce0[o + neke - 2];
    (void)sum_A;
    (void)sum_pz;
  }
  return OMC_OK;
}

void build_ranges(omc_tables *t) {
  int nmed = t->nmed;
  // Maximum cross section per energy loss and its monotonicity.
  for (int imed = 0; imed < nmed; imed++) {
    double sigee = 1.0E-15, sigep = 1.0E-15, sige_old = -1.0, sigp_old = -1.0;
    int ise = 1, isp = 1, neke = t->meke[imed];
    size_t o = static_cast<size_t>(imed) * MXEKE;
    for (int i = 1; i <= neke; i++) {
      double ei = std::exp((static_cast<double>(i) - t->eke0[imed]) / t->eke1[imed]);
      double eil = std::log(ei);
      int leil = i - 1;
      double dedx = t->ededx1[o + leil] * eil + t->ededx0[o + leil];
      double sig = t->esig1[o + leil] * eil + t->esig0[o + leil];
      sig /= dedx;
      if (sig > sigee) sigee = sig;
      if (sig < sige_old) ise = 0;
      sige_old = sig;
      dedx = t->pdedx1[o + leil] * eil + t->pdedx0[o + leil];
      sig = t->psig1[o + leil] * eil + t->psig0[o + leil];
      sig /= dedx;
      if (sig > sigep) sigep = sig;
      if (sig < sigp_old) isp = 0;
      sigp_old = sig;
    }
    t->sig_ismonotone[0 * nmed + imed] = ise;
    t->sig_ismonotone[1 * nmed + imed] = isp;
    t->esig_e[imed] = sigee;
    t->psig_e[imed] = sigep;
  }
  for (int imed = 0; imed < nmed; imed++) {
    size_t o = static_cast<size_t>(imed) * MXEKE;
    double eke0 = t->eke0[imed], eke1 = t->eke1[imed];
    double *rng_e = t->range_ep + 0 * static_cast<size_t>(nmed) * MXEKE + o;
    double *rng_p = t->range_ep + 1 * static_cast<size_t>(nmed) * MXEKE + o;
    double *ea = t->e_array + o;
    // CSDA ranges from the first grid energy (log-interpolated dE/dx and a
    // series expansion of the integral).
    double ei = std::exp((1.0 - eke0) / eke1);
    ea[0] = ei;
    t->expeke1[imed] = std::exp(1.0 / eke1) - 1.0;
    rng_e[0] = 0.0;
    rng_p[0] = 0.0;
    int neke = t->meke[imed];
    for (int i = 1; i <= neke - 1; i++) {
      double eip1 = std::exp((static_cast<double>(i + 1) - eke0) / eke1);
      ea[i] = eip1;
      double eke = 0.5 * (eip1 + ei);
      double elke = std::log(eke);
      int lelke = static_cast<int>(eke1 * elke + eke0) - 1;
      double ededx = t->pdedx1[o + lelke] * elke + t->pdedx0[o + lelke];
      double aux = t->pdedx1[o + i - 1] / ededx;
      rng_p[i] = rng_p[i - 1] + (eip1 - ei) / ededx * (1.0 + aux * (1.0 + 2.0 * aux) * std::pow((eip1 - ei) / eke, 2.0) / 24.0);
      ededx = t->ededx1[o + lelke] * elke + t->ededx0[o + lelke];
      aux = t->ededx1[o + i - 1] / ededx;
      rng_e[i] = rng_e[i - 1] + (eip1 - ei) / ededx * (1.0 + aux * (1.0 + 2.0 * aux) * std::pow(((eip1 - ei) / eke), 2.0) / 24.0);
      ei = eip1;
    }
    // Maximum step (tmxs): the path length over which the energy drops by
    // min(XIMAX * multiple-scattering limit, ESTEPE).
    double eil = (1.0 - eke0) / eke1;
    ei = std::exp(eil);
    int leil = 1;
    double p2 = ei * (ei + 2.0 * kRM);
    double beta2 = p2 / (p2 + std::pow(kRM, 2.0));
    double chi_a2 = t->xcc[imed] / (4.0 * p2 * t->blcc[imed]);
    double dedx0 = t->ededx1[o + leil] * eil + t->ededx0[o + leil];
    double estepx = 2.0 * p2 * beta2 * dedx0 / ei / t->xcc[imed] / (std::log(1.0 + 1.0 / chi_a2) * (1.0 + chi_a2) - 1.0);
    estepx *= XIMAX;
    if (estepx > ESTEPE) estepx = ESTEPE;
    double si = estepx * ei / dedx0;
    for (int i = 1; i <= neke - 1; i++) {
      double elke = (static_cast<double>(i + 1) - eke0) / eke1;
      double eke = std::exp(elke);
      int lelke = i;
      p2 = eke * (eke + 2.0 * kRM);
      beta2 = p2 / (p2 + std::pow(kRM, 2.0));
      chi_a2 = t->xcc[imed] / (4.0 * p2 * t->blcc[imed]);
      double ededx = t->ededx1[o + lelke] * elke + t->ededx0[o + lelke];
      estepx = 2.0 * p2 * beta2 * ededx / eke / (t->xcc[imed]) / (std::log(1.0 + 1.0 / chi_a2) * (1.0 + chi_a2) - 1.0);
      estepx = estepx * XIMAX;
      if (estepx > ESTEPE) estepx = ESTEPE;
      double ekef = (1.0 - estepx) * eke, sip1;
      int lelkef;
      if (ekef <= ea[0]) {
        sip1 = (ea[0] - ekef) / dedx0;
        ekef = ea[0];
        lelkef = 0;
      } else {
        double elkef = std::log(ekef);
        lelkef = static_cast<int>(eke1 * elkef + eke0 - 1);
        int leip1l = lelkef + 1;
        double eip1l = (static_cast<double>(leip1l + 1) - eke0) / eke1;
        double eip1 = ea[leip1l];
        double aux = (eip1 - ekef) / eip1;
        double elktmp = 0.5 * (elkef + eip1l + 0.25 * aux * aux * (1.0 + aux * (1.0 + 0.875 * aux)));
        double ektmp = 0.5 * (ekef + eip1);
        int lelktmp = lelkef;
        ededx = t->ededx1[o + lelktmp] * elktmp + t->ededx0[o + lelktmp];
        aux = t->ededx1[o + lelktmp] / ededx;
        sip1 = (eip1 - ekef) / ededx * (1.0 + aux * (1.0 + 2.0 * aux) * (std::pow(((eip1 - ekef) / ektmp), 2.0) / 24.0));
      }
      sip1 += rng_e[lelke] - rng_e[lelkef + 1];
      t->tmxs1[o + i - 1] = (sip1 - si) * eke1;
      t->tmxs0[o + i - 1] = sip1 - t->tmxs1[o + i - 1] * elke;
      si = sip1;
    }
    t->tmxs0[o + neke - 1] = t->tmxs0[o + neke - 2];
    t->tmxs1[o + neke - 1] = t->tmxs1[o + neke - 2];
  }
}

omc_tables *tables_alloc(int nmed) {
  auto *t = static_cast<omc_tables *>(std::calloc(1, sizeof(omc_tables)));
  if (!t) return nullptr;
  t->nmed = nmed;
  size_t ng = static_cast<size_t>(nmed) * MXGE, ne = static_cast<size_t>(nmed) * MXEKE;
  size_t nr = static_cast<size_t>(nmed) * MXRAYFF;
  size_t nms = static_cast<size_t>(MXL_MS + 1) * (MXQ_MS + 1) * (MXU_MS + 1);
  size_t nspin = static_cast<size_t>(nmed) * 2 * (MXE_SPIN1 + 1) * (MXQ_SPIN + 1) * (MXU_SPIN + 1);
  t->ge0 = dalloc(nmed);
  t->ge1 = dalloc(nmed);
  double **g[] = {&t->gmfp0, &t->gmfp1, &t->gbr10, &t->gbr11, &t->gbr20, &t->gbr21,
                  &t->cohe0, &t->cohe1, &t->pmax0, &t->pmax1};
  for (auto p : g) *p = dalloc(ng);
  double **r[] = {&t->xgrid, &t->fcum, &t->b_array, &t->c_array};
  for (auto p : r) *p = dalloc(nr);
  t->i_array = ialloc(static_cast<size_t>(nmed) * RAYCDFSIZE);
  double **dl[] = {&t->dl1, &t->dl2, &t->dl3, &t->dl4, &t->dl5, &t->dl6};
  for (auto p : dl) *p = dalloc(static_cast<size_t>(nmed) * 8);
  double **pm[] = {&t->bpar0, &t->bpar1, &t->delcm, &t->zbrang, &t->eke0, &t->eke1,
                   &t->esig_e, &t->psig_e, &t->xcc, &t->blcc, &t->expeke1};
  for (auto p : pm) *p = dalloc(nmed);
  double **el[] = {&t->esig0,    &t->esig1,    &t->psig0,    &t->psig1,    &t->ededx0,   &t->ededx1,
                   &t->pdedx0,   &t->pdedx1,   &t->ebr10,    &t->ebr11,    &t->pbr10,    &t->pbr11,
                   &t->pbr20,    &t->pbr21,    &t->tmxs0,    &t->tmxs1,    &t->blcce0,   &t->blcce1,
                   &t->etae_ms0, &t->etae_ms1, &t->etap_ms0, &t->etap_ms1, &t->q1ce_ms0, &t->q1ce_ms1,
                   &t->q1cp_ms0, &t->q1cp_ms1, &t->q2ce_ms0, &t->q2ce_ms1, &t->q2cp_ms0, &t->q2cp_ms1,
                   &t->e_array};
  for (auto p : el) *p = dalloc(ne);
  t->range_ep = dalloc(2 * ne);
  t->sig_ismonotone = ialloc(2 * static_cast<size_t>(nmed));
  t->spin_rej = dalloc(nspin);
  t->ums = dalloc(nms);
  t->fms = dalloc(nms);
  t->wms = dalloc(nms);
  t->ims = ialloc(nms);
  return t;
}

}  // namespace

extern "C" void omc_tables_free(omc_tables *t) {
  if (!t) return;
  void *ptrs[] = {t->ge0,      t->ge1,      t->gmfp0,    t->gmfp1,    t->gbr10,    t->gbr11,    t->gbr20,
                  t->gbr21,    t->cohe0,    t->cohe1,    t->xgrid,    t->fcum,     t->b_array,  t->c_array,
                  t->pmax0,    t->pmax1,    t->i_array,  t->dl1,      t->dl2,      t->dl3,      t->dl4,
                  t->dl5,      t->dl6,      t->bpar0,    t->bpar1,    t->delcm,    t->zbrang,   t->esig0,
                  t->esig1,    t->psig0,    t->psig1,    t->ededx0,   t->ededx1,   t->pdedx0,   t->pdedx1,
                  t->ebr10,    t->ebr11,    t->pbr10,    t->pbr11,    t->pbr20,    t->pbr21,    t->tmxs0,
                  t->tmxs1,    t->blcce0,   t->blcce1,   t->etae_ms0, t->etae_ms1, t->etap_ms0, t->etap_ms1,
                  t->q1ce_ms0, t->q1ce_ms1, t->q1cp_ms0, t->q1cp_ms1, t->q2ce_ms0, t->q2ce_ms1, t->q2cp_ms0,
                  t->q2cp_ms1, t->e_array,  t->range_ep, t->eke0,     t->eke1,     t->sig_ismonotone,
                  t->esig_e,   t->psig_e,   t->xcc,      t->blcc,     t->expeke1,  t->spin_rej, t->ums,
                  t->fms,      t->wms,      t->ims};
  for (void *p : ptrs) std::free(p);
  std::free(t);
}

extern "C" omc_status omc_tables_build(const omc_input *in, int nmed, const char (*med_names)[OMC_NAME_LEN],
                                       omc_tables **out) {
  if (!in || !med_names || !out) return fail(OMC_ERR_ARG, "null argument");
  if (nmed < 1 || nmed > OMC_MXMED) return fail(OMC_ERR_ARG, "nmed %d outside 1..%d", nmed, OMC_MXMED);
  char buf[1024];
  if (!omc_input_get(in, "pegs file", buf, sizeof buf))
    return fail(OMC_ERR_INPUT, "Can not find 'pegs file' key on input file.");
  std::string pegs = omc::remove_spaces(buf);
  if (!omc_input_get(in, "pgs4form file", buf, sizeof buf))
    return fail(OMC_ERR_INPUT, "Can not find 'pgs4form file' key on input file.");
  std::string pgs4form = omc::remove_spaces(buf);
  if (!omc_input_get(in, "data folder", buf, sizeof buf))
    return fail(OMC_ERR_INPUT, "Can not find 'data folder' key on input file.");
  std::string folder = omc::remove_spaces(buf);
  omc_tables *t = tables_alloc(nmed);
  if (!t) return fail(OMC_ERR_NOMEM, "table allocation failed");
  for (int i = 0; i < nmed; i++) std::strncpy(t->names[i], med_names[i], OMC_NAME_LEN - 1);
  std::vector<Medium> media(nmed);
  omc_status s;
  if ((s = read_pegs(pegs, t, media)) != OMC_OK || (s = build_photon(t, media, folder)) != OMC_OK ||
      (s = build_rayleigh(t, media, pgs4form)) != OMC_OK) {
    omc_tables_free(t);
    return s;
  }
  build_pair(t, media);
  if ((s = read_msnew(t, folder + "msnew.data")) != OMC_OK) {
    omc_tables_free(t);
    return s;
  }
  for (int i = 0; i < nmed; i++) {
    t->blcc[i] = 1.16699413758864573 * t->blcc[i];  // Euler constant absorbed
    t->xcc[i] = std::pow(t->xcc[i], 2.0);
  }
  if ((s = build_spin(t, media, folder + "spinms.data")) != OMC_OK) {
    omc_tables_free(t);
    return s;
  }
  build_ranges(t);
  *out = t;
  return OMC_OK;
}

// ---------------------------------------------------------------------------
// Dump in the oracle's record format.
// ---------------------------------------------------------------------------
namespace {
struct Dump {
  FILE *f;
  void arr(const char *name, char type, const void *p, uint64_t n) {
    uint32_t len = static_cast<uint32_t>(std::strlen(name));
    std::fwrite(&len, 4, 1, f);
    std::fwrite(name, 1, len, f);
    std::fwrite(&type, 1, 1, f);
    std::fwrite(&n, 8, 1, f);
    if (n) std::fwrite(p, type == 'd' ? 8 : 4, n, f);
  }
  void d(const char *name, const double *p, uint64_t n) { arr(name, 'd', p, n); }
  void i(const char *name, const int *p, uint64_t n) { arr(name, 'i', p, n); }
  void s(const char *name, double v) { arr(name, 'd', &v, 1); }
};
}  // namespace

extern "C" omc_status omc_tables_dump(const omc_tables *t, const char *path) {
  if (!t || !path) return fail(OMC_ERR_ARG, "null argument");
  FILE *f = std::fopen(path, "wb");
  if (!f) return fail(OMC_ERR_IO, "Unable to open file: %s", path);
  std::fwrite("OMCT", 1, 4, f);
  Dump d{f};
  int n = t->nmed;
  uint64_t ng = static_cast<uint64_t>(n) * MXGE, ne = static_cast<uint64_t>(n) * MXEKE;
  uint64_t nr = static_cast<uint64_t>(n) * MXRAYFF;
  d.s("nmed", n);
  d.d("pegs.rho", t->rho, n);
  d.d("pegs.rlc", t->rlc, n);
  d.d("pegs.ae", t->ae, n);
  d.d("pegs.ap", t->ap, n);
  d.d("pegs.ue", t->ue, n);
  d.d("pegs.up", t->up, n);
  d.d("pegs.te", t->te, n);
  d.d("pegs.thmoll", t->thmoll, n);
  d.d("pegs.delcm", t->pegs_delcm, n);
  d.i("pegs.meke", t->meke, n);
  d.i("pegs.ne", t->ne, n);
  d.d("photon.ge0", t->ge0, n);
  d.d("photon.ge1", t->ge1, n);
  d.d("photon.gmfp0", t->gmfp0, ng);
  d.d("photon.gmfp1", t->gmfp1, ng);
  d.d("photon.gbr10", t->gbr10, ng);
  d.d("photon.gbr11", t->gbr11, ng);
  d.d("photon.gbr20", t->gbr20, ng);
  d.d("photon.gbr21", t->gbr21, ng);
  d.d("photon.cohe0", t->cohe0, ng);
  d.d("photon.cohe1", t->cohe1, ng);
  d.d("rayleigh.xgrid", t->xgrid, nr);
  d.d("rayleigh.fcum", t->fcum, nr);
  d.d("rayleigh.b_array", t->b_array, nr);
  d.d("rayleigh.c_array", t->c_array, nr);
  d.i("rayleigh.i_array", t->i_array, nr);
  d.d("rayleigh.pmax0", t->pmax0, ng);
  d.d("rayleigh.pmax1", t->pmax1, ng);
  d.d("pair.dl1", t->dl1, 8 * n);
  d.d("pair.dl2", t->dl2, 8 * n);
  d.d("pair.dl3", t->dl3, 8 * n);
  d.d("pair.dl4", t->dl4, 8 * n);
  d.d("pair.dl5", t->dl5, 8 * n);
  d.d("pair.dl6", t->dl6, 8 * n);
  d.d("pair.bpar0", t->bpar0, n);
  d.d("pair.bpar1", t->bpar1, n);
  d.d("pair.delcm", t->delcm, n);
  d.d("pair.zbrang", t->zbrang, n);
#define ELEC(field) d.d("electron." #field, t->field, ne);
  ELEC(esig0) ELEC(esig1) ELEC(psig0) ELEC(psig1) ELEC(ededx0) ELEC(ededx1) ELEC(pdedx0) ELEC(pdedx1)
  ELEC(ebr10) ELEC(ebr11) ELEC(pbr10) ELEC(pbr11) ELEC(pbr20) ELEC(pbr21) ELEC(tmxs0) ELEC(tmxs1)
  ELEC(blcce0) ELEC(blcce1) ELEC(etae_ms0) ELEC(etae_ms1) ELEC(etap_ms0) ELEC(etap_ms1)
  ELEC(q1ce_ms0) ELEC(q1ce_ms1) ELEC(q1cp_ms0) ELEC(q1cp_ms1) ELEC(q2ce_ms0) ELEC(q2ce_ms1)
  ELEC(q2cp_ms0) ELEC(q2cp_ms1) ELEC(e_array)
#undef ELEC
  d.d("electron.range_ep", t->range_ep, 2 * ne);
  d.d("electron.eke0", t->eke0, n);
  d.d("electron.eke1", t->eke1, n);
  d.i("electron.sig_ismonotone", t->sig_ismonotone, 2 * n);
  d.d("electron.esig_e", t->esig_e, n);
  d.d("electron.psig_e", t->psig_e, n);
  d.d("electron.xcc", t->xcc, n);
  d.d("electron.blcc", t->blcc, n);
  d.d("electron.expeke1", t->expeke1, n);
  d.s("spin.b2spin_min", t->b2spin_min);
  d.s("spin.dbeta2i", t->dbeta2i);
  d.s("spin.espml", t->espml);
  d.s("spin.dleneri", t->dleneri);
  d.s("spin.dqq1i", t->dqq1i);
  d.d("spin.spin_rej", t->spin_rej,
      static_cast<uint64_t>(n) * 2 * (MXE_SPIN1 + 1) * (MXQ_SPIN + 1) * (MXU_SPIN + 1));
  uint64_t nm = static_cast<uint64_t>(MXL_MS + 1) * (MXQ_MS + 1) * (MXU_MS + 1);
  d.d("mscat.ums", t->ums, nm);
  d.d("mscat.fms", t->fms, nm);
  d.d("mscat.wms", t->wms, nm);
  d.i("mscat.ims", t->ims, nm);
  d.s("mscat.dllambi", t->dllambi);
  d.s("mscat.dqmsi", t->dqmsi);
  std::fclose(f);
  return OMC_OK;
}
