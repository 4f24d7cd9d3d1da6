// Host side of the C ABI: input file, phantom, regions, source and scoring
// output.  Each function restates the reference user-code routine named in
// its comment; the interaction tables live in media.cpp.
#include <algorithm>
#include <cctype>
#include <charconv>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "common.h"

using omc::fail;

// ---------------------------------------------------------------------------
// Input file: parseInputFile / getInputValue (omc_utilities.c:63-123).
// ---------------------------------------------------------------------------
struct omc_input {
  std::vector<std::pair<std::string, std::string>> items;
};

static bool line_blank(const std::string &s) {
  for (char c : s)
    if (!std::isspace(static_cast<unsigned char>(c))) return false;
  return true;
}

static omc_status parse_text(const std::string &text, omc_input **out) {
  auto *in = new omc_input();
  for (const std::string &line : omc::split_lines(text)) {
    // Lines holding '#' anywhere, and blank lines, are skipped.
    if (line.find('#') != std::string::npos || line_blank(line)) continue;
    // key = first token delimited by '=', value = the rest of the line.
    size_t k0 = line.find_first_not_of('=');
    if (k0 == std::string::npos) continue;
    size_t eq = line.find('=', k0);
    std::string key = line.substr(k0, eq == std::string::npos ? std::string::npos : eq - k0);
    std::string value;
    if (eq != std::string::npos) {
      size_t v0 = eq + 1;
      value = line.substr(v0);
    }
    in->items.emplace_back(key, value);
  }
  *out = in;
  return OMC_OK;
}

extern "C" omc_status omc_input_parse(const char *path_without_ext, omc_input **out) {
  if (!path_without_ext || !out) return fail(OMC_ERR_ARG, "null argument");
  std::string path = std::string(path_without_ext) + ".inp";
  std::string text;
  if (!omc::read_file(path, text)) return fail(OMC_ERR_IO, "Unable to open file: %s", path.c_str());
  return parse_text(text, out);
}

extern "C" omc_status omc_input_from_string(const char *text, omc_input **out) {
  if (!text || !out) return fail(OMC_ERR_ARG, "null argument");
  return parse_text(text, out);
}

extern "C" int omc_input_get(const omc_input *in, const char *key, char *dest, size_t cap) {
  if (!in || !key) return 0;
  for (const auto &kv : in->items) {
    if (kv.first.find(key) != std::string::npos) {  // substring match
      if (dest && cap) {
        size_t n = kv.second.size() < cap - 1 ? kv.second.size() : cap - 1;
        std::memcpy(dest, kv.second.data(), n);
        dest[n] = '\0';
      }
      return 1;
    }
  }
  return 0;
}

extern "C" void omc_input_free(omc_input *in) { delete in; }

static bool get_value(const omc_input *in, const char *key, std::string &v) {
  char buf[1024];
  if (!omc_input_get(in, key, buf, sizeof buf)) return false;
  v = buf;
  return true;
}

// ---------------------------------------------------------------------------
// Phantom: initPhantom (omc_dosxyz.c:62-175).
// ---------------------------------------------------------------------------
static omc_phantom *phantom_alloc(int nx, int ny, int nz) {
  auto *ph = static_cast<omc_phantom *>(std::calloc(1, sizeof(omc_phantom)));
  if (!ph) return nullptr;
  size_t nv = static_cast<size_t>(nx) * ny * nz;
  ph->nx = nx;
  ph->ny = ny;
  ph->nz = nz;
  ph->xbounds = static_cast<double *>(std::malloc((nx + 1) * sizeof(double)));
  ph->ybounds = static_cast<double *>(std::malloc((ny + 1) * sizeof(double)));
  ph->zbounds = static_cast<double *>(std::malloc((nz + 1) * sizeof(double)));
  ph->med_index = static_cast<int *>(std::malloc(nv * sizeof(int)));
  ph->density = static_cast<double *>(std::malloc(nv * sizeof(double)));
  if (!ph->xbounds || !ph->ybounds || !ph->zbounds || !ph->med_index || !ph->density) {
    omc_phantom_free(ph);
    return nullptr;
  }
  return ph;
}

extern "C" void omc_phantom_free(omc_phantom *ph) {
  if (!ph) return;
  std::free(ph->xbounds);
  std::free(ph->ybounds);
  std::free(ph->zbounds);
  std::free(ph->med_index);
  std::free(ph->density);
  std::free(ph);
}

namespace {

bool is_space(char c) { return std::isspace(static_cast<unsigned char>(c)) != 0; }

// The first n whitespace-separated numbers of [begin, end) (NUL at end) into
// out, each converted by strtod as fscanf's %lf does; false if the text
// holds fewer, or a token that is not a number comes first.  Large blocks
// are cut at whitespace into one piece per thread, parsed in parallel and
// joined in order, which gives the sequential result.
bool parse_numbers(const char *begin, const char *end, double *out, size_t n) {
  const size_t bytes = static_cast<size_t>(end - begin);
  unsigned hw = std::thread::hardware_concurrency();
  size_t nthreads = std::max<size_t>(1, std::min<size_t>(hw ? hw : 1, 32));
  if (bytes < (1u << 20)) nthreads = 1;
  std::vector<const char *> cut(nthreads + 1, end);
  cut[0] = begin;
  for (size_t t = 1; t < nthreads; t++) {
    const char *c = std::max(cut[t - 1], begin + bytes / nthreads * t);
    while (c < end && !is_space(*c)) c++;  // a piece never splits a token
    cut[t] = c;
  }
  struct Piece {
    std::vector<double> v;
    bool stopped = false;  // a token that is not a number ended the piece
  };
  std::vector<Piece> parts(nthreads);
  auto work = [&](size_t t) {
    Piece &pc = parts[t];
    pc.v.reserve(static_cast<size_t>(cut[t + 1] - cut[t]) / 4 + 16);
    const char *p = cut[t];
    const char *stop = cut[t + 1];
    for (;;) {
      while (p < stop && is_space(*p)) p++;
      if (p >= stop) return;
      // from_chars and strtod both round correctly; from_chars is taken
      // only where it reads the whole token (no '+', hex or range error).
      double x = 0;
      auto r = std::from_chars(p, stop, x);
      if (r.ec == std::errc() && (r.ptr == stop || is_space(*r.ptr))) {
        pc.v.push_back(x);
        p = r.ptr;
        continue;
      }
      char *e = nullptr;
      x = std::strtod(p, &e);
      if (e == p) {
        pc.stopped = true;
        return;
      }
      pc.v.push_back(x);
      p = e;
    }
  };
  auto run = [nthreads](const auto &fn) {
    std::vector<std::thread> th;
    for (size_t t = 1; t < nthreads; t++) th.emplace_back(fn, t);
    fn(0);
    for (auto &t : th) t.join();
  };
  run(work);
  // Join in order: piece t supplies values [at[t], at[t] + take[t]).
  std::vector<size_t> at(nthreads, 0), take(nthreads, 0);
  size_t got = 0;
  bool ok = false;
  for (size_t t = 0; t < nthreads && !ok; t++) {
    at[t] = got;
    take[t] = std::min(parts[t].v.size(), n - got);
    got += take[t];
    if (got == n) ok = true;
    else if (parts[t].stopped) break;
  }
  if (!ok) return false;
  run([&](size_t t) {
    std::copy(parts[t].v.begin(), parts[t].v.begin() + static_cast<std::ptrdiff_t>(take[t]), out + at[t]);
  });
  return true;
}

}  // namespace

extern "C" omc_status omc_phantom_read(const char *path, omc_phantom **out) {
  if (!path || !out) return fail(OMC_ERR_ARG, "null argument");
  std::string text;
  if (!omc::read_file(path, text)) return fail(OMC_ERR_IO, "Unable to open file: %s", path);
  // Line-oriented header: nmed, media names, a dummy line, then nx ny nz.
  size_t pos = 0;
  auto next_line = [&](std::string &line) -> bool {
    if (pos >= text.size()) return false;
    size_t nl = text.find('\n', pos);
    if (nl == std::string::npos) nl = text.size();
    line = text.substr(pos, nl - pos);
    pos = nl + 1;
    return true;
  };
  std::string line;
  if (!next_line(line)) return fail(OMC_ERR_FORMAT, "%s: empty phantom file", path);
  int nmed = std::atoi(line.c_str());
  if (nmed < 1 || nmed > OMC_MXMED)
    return fail(OMC_ERR_FORMAT, "%s: number of media %d outside 1..%d", path, nmed, OMC_MXMED);
  char names[OMC_MXMED][OMC_NAME_LEN] = {};
  for (int i = 0; i < nmed; i++) {
    if (!next_line(line)) return fail(OMC_ERR_FORMAT, "%s: missing medium name", path);
    std::string n = omc::remove_spaces(line);
    std::strncpy(names[i], n.c_str(), OMC_NAME_LEN - 1);
  }
  if (!next_line(line)) return fail(OMC_ERR_FORMAT, "%s: truncated header", path);  // dummy line
  if (!next_line(line)) return fail(OMC_ERR_FORMAT, "%s: truncated header", path);
  int nx = 0, ny = 0, nz = 0;
  if (std::sscanf(line.c_str(), "%d %d %d", &nx, &ny, &nz) != 3 || nx < 1 || ny < 1 || nz < 1)
    return fail(OMC_ERR_FORMAT, "%s: bad voxel counts", path);
  omc_phantom *ph = phantom_alloc(nx, ny, nz);
  if (!ph) return fail(OMC_ERR_NOMEM, "phantom allocation failed");
  ph->nmed = nmed;
  std::memcpy(ph->med_names, names, sizeof names);
  // Bounds: whitespace-separated numbers (fscanf %lf), then the rest of the
  // line holding the last z bound is skipped.
  omc::NumberStream ns(text.c_str() + pos);
  auto read_bounds = [&](double *b, int n) {
    for (int i = 0; i <= n; i++)
      if (!ns.next(b[i])) return false;
    return true;
  };
  if (!read_bounds(ph->xbounds, nx) || !read_bounds(ph->ybounds, ny) || !read_bounds(ph->zbounds, nz)) {
    omc_phantom_free(ph);
    return fail(OMC_ERR_FORMAT, "%s: truncated voxel bounds", path);
  }
  pos = static_cast<size_t>(ns.pos() - text.c_str());
  next_line(line);
  // Media: one character per voxel, one row of nx per line, a blank line
  // after every z slice.
  for (int k = 0; k < nz; k++) {
    for (int j = 0; j < ny; j++) {
      if (pos + nx > text.size()) {
        omc_phantom_free(ph);
        return fail(OMC_ERR_FORMAT, "%s: truncated media block", path);
      }
      for (int i = 0; i < nx; i++) {
        size_t irl = i + static_cast<size_t>(j) * nx + static_cast<size_t>(k) * ny * nx;
        ph->med_index[irl] = text[pos + i] - '0';
      }
      pos += nx;
      next_line(line);  // rest of the row
    }
    next_line(line);  // blank line
  }
  // Densities: whitespace-separated numbers in region order, the first nv
  // of them.
  size_t nv = static_cast<size_t>(nx) * ny * nz;
  if (!parse_numbers(text.c_str() + (pos < text.size() ? pos : text.size()),
                     text.c_str() + text.size(), ph->density, nv)) {
    omc_phantom_free(ph);
    return fail(OMC_ERR_FORMAT, "%s: truncated density block", path);
  }
  for (size_t v = 0; v < nv; v++) {
    if (ph->med_index[v] < 0 || ph->med_index[v] > nmed) {
      omc_phantom_free(ph);
      return fail(OMC_ERR_FORMAT, "%s: medium index %d outside 0..%d", path, ph->med_index[v], nmed);
    }
  }
  *out = ph;
  return OMC_OK;
}

extern "C" omc_status omc_phantom_create(int nmed, const char *const *med_names, int nx, int ny, int nz,
                                         const double *xb, const double *yb, const double *zb,
                                         const int *med_index, const double *density, omc_phantom **out) {
  if (!out || !med_names || !xb || !yb || !zb || !med_index || !density)
    return fail(OMC_ERR_ARG, "null argument");
  if (nmed < 1 || nmed > OMC_MXMED) return fail(OMC_ERR_ARG, "nmed %d outside 1..%d", nmed, OMC_MXMED);
  if (nx < 1 || ny < 1 || nz < 1) return fail(OMC_ERR_ARG, "bad voxel counts");
  omc_phantom *ph = phantom_alloc(nx, ny, nz);
  if (!ph) return fail(OMC_ERR_NOMEM, "phantom allocation failed");
  ph->nmed = nmed;
  for (int i = 0; i < nmed; i++) std::strncpy(ph->med_names[i], med_names[i], OMC_NAME_LEN - 1);
  std::memcpy(ph->xbounds, xb, (nx + 1) * sizeof(double));
  std::memcpy(ph->ybounds, yb, (ny + 1) * sizeof(double));
  std::memcpy(ph->zbounds, zb, (nz + 1) * sizeof(double));
  size_t nv = static_cast<size_t>(nx) * ny * nz;
  for (size_t v = 0; v < nv; v++) {
    if (med_index[v] < 0 || med_index[v] > nmed) {
      omc_phantom_free(ph);
      return fail(OMC_ERR_ARG, "medium index %d outside 0..%d", med_index[v], nmed);
    }
  }
  std::memcpy(ph->med_index, med_index, nv * sizeof(int));
  std::memcpy(ph->density, density, nv * sizeof(double));
  *out = ph;
  return OMC_OK;
}

extern "C" omc_status omc_phantom_write(const omc_phantom *ph, const char *path) {
  if (!ph || !path) return fail(OMC_ERR_ARG, "null argument");
  FILE *f = std::fopen(path, "w");
  if (!f) return fail(OMC_ERR_IO, "Unable to open file: %s", path);
  std::fprintf(f, "%d\n", ph->nmed);
  for (int i = 0; i < ph->nmed; i++) std::fprintf(f, "%s\n", ph->med_names[i]);
  for (int i = 0; i < ph->nmed; i++) std::fprintf(f, "  0.25");
  std::fprintf(f, "\n%d %d %d\n", ph->nx, ph->ny, ph->nz);
  auto bounds = [&](const double *b, int n) {
    for (int i = 0; i <= n; i++) std::fprintf(f, "%.17g%s", b[i], (i % 8 == 7 || i == n) ? "\n" : " ");
  };
  bounds(ph->xbounds, ph->nx);
  bounds(ph->ybounds, ph->ny);
  bounds(ph->zbounds, ph->nz);
  std::vector<char> row(ph->nx + 1);
  for (int k = 0; k < ph->nz; k++) {
    for (int j = 0; j < ph->ny; j++) {
      for (int i = 0; i < ph->nx; i++) {
        size_t v = i + static_cast<size_t>(j) * ph->nx + static_cast<size_t>(k) * ph->nx * ph->ny;
        row[i] = static_cast<char>('0' + ph->med_index[v]);
      }
      row[ph->nx] = '\0';
      std::fprintf(f, "%s\n", row.data());
    }
    std::fprintf(f, "\n");
  }
  for (int k = 0; k < ph->nz; k++) {
    for (int j = 0; j < ph->ny; j++) {
      for (int i = 0; i < ph->nx; i++) {
        size_t v = i + static_cast<size_t>(j) * ph->nx + static_cast<size_t>(k) * ph->nx * ph->ny;
        std::fprintf(f, "%.17g ", ph->density[v]);
      }
      std::fprintf(f, "\n");
    }
    std::fprintf(f, "\n");
  }
  std::fclose(f);
  return OMC_OK;
}

// ---------------------------------------------------------------------------
// Regions: initRegions (omc_dosxyz.c:890-962).
// ---------------------------------------------------------------------------
extern "C" void omc_regions_free(omc_regions *r) {
  if (!r) return;
  std::free(r->med);
  std::free(r->rhof);
  std::free(r->pcut);
  std::free(r->ecut);
  std::free(r);
}

extern "C" omc_status omc_regions_build(const omc_input *in, const omc_phantom *ph, const omc_tables *t,
                                        omc_regions **out) {
  if (!in || !ph || !t || !out) return fail(OMC_ERR_ARG, "null argument");
  std::string v;
  if (!get_value(in, "global ecut", v)) return fail(OMC_ERR_INPUT, "Can not find 'global ecut' key on input file.");
  double ecut = std::atof(v.c_str());
  if (!get_value(in, "global pcut", v)) return fail(OMC_ERR_INPUT, "Can not find 'global pcut' key on input file.");
  double pcut = std::atof(v.c_str());
  int nreg = ph->nx * ph->ny * ph->nz + 1;
  auto *r = static_cast<omc_regions *>(std::calloc(1, sizeof(omc_regions)));
  r->nreg = nreg;
  r->med = static_cast<int *>(std::calloc(nreg, sizeof(int)));
  r->rhof = static_cast<double *>(std::calloc(nreg, sizeof(double)));
  r->pcut = static_cast<double *>(std::calloc(nreg, sizeof(double)));
  r->ecut = static_cast<double *>(std::calloc(nreg, sizeof(double)));
  if (!r->med || !r->rhof || !r->pcut || !r->ecut) {
    omc_regions_free(r);
    return fail(OMC_ERR_NOMEM, "region allocation failed");
  }
  r->med[0] = -1;  // region 0: outside the phantom
  for (int i = 1; i < nreg; i++) {
    int imed = ph->med_index[i - 1] - 1;
    r->med[i] = imed;
    if (imed == -1) continue;  // vacuum voxel: rhof/pcut/ecut stay 0
    if (imed >= t->nmed) {
      omc_regions_free(r);
      return fail(OMC_ERR_ARG, "region %d uses medium %d but tables hold %d media", i, imed + 1, t->nmed);
    }
    double rho = ph->density[i - 1];
    r->rhof[i] = (rho == 0.0) ? 1.0 : rho / t->rho[imed];
    r->pcut[i] = (t->ap[imed] <= pcut) ? pcut : t->ap[imed];
    r->ecut[i] = (t->ae[imed] <= ecut) ? ecut : t->ae[imed];
  }
  *out = r;
  return OMC_OK;
}

// ---------------------------------------------------------------------------
// Source: initSource (omc_dosxyz.c:368-632).
// ---------------------------------------------------------------------------
extern "C" void omc_source_free(omc_source *s) { std::free(s); }

extern "C" omc_status omc_source_build(const omc_input *in, const omc_phantom *ph, omc_source **out) {
  if (!in || !ph || !out) return fail(OMC_ERR_ARG, "null argument");
  auto *s = static_cast<omc_source *>(std::calloc(1, sizeof(omc_source)));
  if (!s) return fail(OMC_ERR_NOMEM, "source allocation failed");
  std::string v;
  s->spectrum = get_value(in, "spectrum file", v) ? 1 : 0;
  if (s->spectrum) {
    std::string path = omc::remove_spaces(v), text;
    if (!omc::read_file(path, text)) {
      omc_source_free(s);
      return fail(OMC_ERR_IO, "Unable to open file: %s", path.c_str());
    }
    std::vector<std::string> lines = omc::split_lines(text);
    int nensrc = 0, imode = 0;
    double enmin = 0.0;
    if (lines.size() < 2 || std::sscanf(lines[1].c_str(), "%d %lf %d", &nensrc, &enmin, &imode) != 3) {
      omc_source_free(s);
      return fail(OMC_ERR_FORMAT, "%s: bad spectrum header", path.c_str());
    }
    if (nensrc > OMC_MXEBIN || nensrc < 1 || lines.size() < static_cast<size_t>(2 + nensrc)) {
      omc_source_free(s);
      return fail(OMC_ERR_FORMAT, "%s: number of energy bins %d invalid (max %d)", path.c_str(), nensrc, OMC_MXEBIN);
    }
    std::vector<double> ensrcd(nensrc), srcpdf(nensrc), srccdf(nensrc);
    for (int i = 0; i < nensrc; i++) {
      if (std::sscanf(lines[2 + i].c_str(), "%lf %lf", &ensrcd[i], &srcpdf[i]) != 2) {
        omc_source_free(s);
        return fail(OMC_ERR_FORMAT, "%s: bad spectrum row %d", path.c_str(), i);
      }
    }
    if (imode == 1) {  // counts/MeV -> counts/bin
      srcpdf[0] *= (ensrcd[0] - enmin);
      for (int i = 1; i < nensrc; i++) srcpdf[i] *= (ensrcd[i] - ensrcd[i - 1]);
    } else if (imode != 0) {
      omc_source_free(s);
      return fail(OMC_ERR_FORMAT, "Invalid mode number in spectrum file.");
    }
    // Inverse CDF on INVDIM bins (omc_dosxyz.c:447-503).
    srccdf[0] = srcpdf[0];
    for (int i = 1; i < nensrc; i++) srccdf[i] = srccdf[i - 1] + srcpdf[i];
    double fnorm = 1.0 / srccdf[nensrc - 1];
    s->deltak = OMC_INVDIM;
    double gridsz = 1.0f / s->deltak;
    for (int i = 0; i < nensrc; i++) srccdf[i] *= fnorm;
    for (int k = 0; k < OMC_INVDIM; k++) {
      double ak = static_cast<double>(k) * gridsz;
      int i = 0;
      while (i < nensrc && !(ak <= srccdf[i])) i++;
      if (i >= nensrc) i = nensrc - 1;  // cdf round-off above 1
      s->cdfinv1[k] = (i != 0) ? ensrcd[i - 1] : enmin;
      s->cdfinv2[k] = ensrcd[i] - s->cdfinv1[k];
    }
  } else {
    if (!get_value(in, "mono energy", v)) {
      omc_source_free(s);
      return fail(OMC_ERR_INPUT, "Can not find 'mono energy' key on input file.");
    }
    s->energy = std::atof(v.c_str());
  }
  if (!get_value(in, "collimator bounds", v) ||
      std::sscanf(v.c_str(), "%lf %lf %lf %lf", &s->xinl, &s->xinu, &s->yinl, &s->yinu) != 4) {
    omc_source_free(s);
    return fail(OMC_ERR_INPUT, "Can not find 'collimator bounds' key on input file.");
  }
  const double *xb = ph->xbounds, *yb = ph->ybounds;
  int nx = ph->nx, ny = ph->ny;
  // x range clipped to the phantom, then the voxel index range it covers.
  if (s->xinl < xb[0]) s->xinl = xb[0];
  if (s->xinu <= s->xinl) s->xinu = s->xinl;
  if (s->xinu > xb[nx]) s->xinu = xb[nx];
  if (s->xinl > xb[nx]) s->xinl = xb[nx];
  s->ixinl = 0;
  while (s->ixinl < nx - 1 && xb[s->ixinl] <= s->xinl && xb[s->ixinl + 1] < s->xinl) s->ixinl++;
  s->ixinu = s->ixinl - 1;
  while (s->ixinu < nx - 1 && (s->ixinu < 0 || xb[s->ixinu] <= s->xinu) && xb[s->ixinu + 1] < s->xinu) s->ixinu++;
  if (s->yinl < yb[0]) s->yinl = yb[0];
  if (s->yinu <= s->yinl) s->yinu = s->yinl;
  if (s->yinu > yb[ny]) s->yinu = yb[ny];
  if (s->yinl > yb[ny]) s->yinl = yb[ny];
  s->iyinl = 0;
  while (s->iyinl < ny - 1 && yb[s->iyinl] <= s->yinl && yb[s->iyinl + 1] < s->yinl) s->iyinl++;
  s->iyinu = s->iyinl - 1;
  while (s->iyinu < ny - 1 && (s->iyinu < 0 || yb[s->iyinu] <= s->yinu) && yb[s->iyinu + 1] < s->yinu) s->iyinu++;
  s->xsize = s->xinu - s->xinl;
  s->ysize = s->yinu - s->yinl;
  if (!get_value(in, "charge", v)) {
    omc_source_free(s);
    return fail(OMC_ERR_INPUT, "Can not find 'charge' key on input file.");
  }
  s->charge = std::atoi(v.c_str());
  if (s->charge < -1 || s->charge > 1) {
    omc_source_free(s);
    return fail(OMC_ERR_INPUT, "Particle kind not recognized.");
  }
  if (!get_value(in, "ssd", v)) {
    omc_source_free(s);
    return fail(OMC_ERR_INPUT, "Can not find 'ssd' key on input file.");
  }
  s->ssd = std::atof(v.c_str());
  if (s->ssd < 0) {
    omc_source_free(s);
    return fail(OMC_ERR_INPUT, "SSD must be greater than zero.");
  }
  *out = s;
  return OMC_OK;
}

// ---------------------------------------------------------------------------
// Scoring output: accumulateResults / outputResults (omc_dosxyz.c:719-886).
// ---------------------------------------------------------------------------
extern "C" omc_status omc_accumulate_results(const omc_phantom *ph, const double *accum_endep,
                                             const double *accum_endep2, int iout, long long nhist,
                                             int nbatch, double *dose, double *unc) {
  if (!ph || !accum_endep || !accum_endep2 || !dose || !unc) return fail(OMC_ERR_ARG, "null argument");
  if (nbatch < 2) return fail(OMC_ERR_ARG, "batch statistics need nbatch >= 2");
  int nx = ph->nx, ny = ph->ny, nz = ph->nz;
  double inc_fluence = static_cast<double>(nhist);
  dose[0] = 0.0;
  unc[0] = 0.0;
  for (int iz = 0; iz < nz; iz++)
    for (int iy = 0; iy < ny; iy++)
      for (int ix = 0; ix < nx; ix++) {
        size_t irl = 1 + ix + static_cast<size_t>(iy) * nx + static_cast<size_t>(iz) * nx * ny;
        double endep = accum_endep[irl] / static_cast<double>(nbatch);
        double endep2 = accum_endep2[irl] / static_cast<double>(nbatch);
        double u;
        if (endep != 0.0) {
          u = endep2 - endep * endep;
          u /= static_cast<double>(nbatch - 1);
          u = std::sqrt(u) / endep;
        } else {
          endep = 0.0;
          u = 0.9999999;
        }
        if (iout) {
          double mass = (ph->xbounds[ix + 1] - ph->xbounds[ix]) * (ph->ybounds[iy + 1] - ph->ybounds[iy]) *
                        (ph->zbounds[iz + 1] - ph->zbounds[iz]);
          mass *= ph->density[irl - 1];
          endep *= 1.602E-10 / (mass * inc_fluence);
        } else {
          endep /= inc_fluence;
        }
        if (ph->density[irl - 1] < 0.044) {  // zero dose in air
          endep = 0.0;
          u = 0.9999999;
        }
        dose[irl] = endep;
        unc[irl] = u;
      }
  return OMC_OK;
}

namespace {

// n values as "<value> " each (precision 6, the given format), then '\n'.
bool write_formatted(FILE *f, const double *v, size_t n, std::chars_format fmt) {
  unsigned hw = std::thread::hardware_concurrency();
  size_t nthreads = std::max<size_t>(1, std::min<size_t>(hw ? hw : 1, 32));
  if (n < (1u << 16)) nthreads = 1;
  size_t per = (n + nthreads - 1) / nthreads;
  std::vector<std::string> parts(nthreads);
  auto work = [&](size_t t) {
    size_t lo = t * per, hi = std::min(n, lo + per);
    std::string &out = parts[t];
    out.resize((hi > lo ? hi - lo : 0) * 16);
    char *p = out.data(), *end = out.data() + out.size();
    for (size_t i = lo; i < hi; i++) {
      auto r = std::to_chars(p, end, v[i], fmt, 6);
      p = r.ptr;
      *p++ = ' ';
      if (end - p < 400) {  // room for the longest fixed-format double
        size_t used = static_cast<size_t>(p - out.data());
        out.resize(out.size() * 2 + 1024);
        p = out.data() + used;
        end = out.data() + out.size();
      }
    }
    out.resize(static_cast<size_t>(p - out.data()));
  };
  std::vector<std::thread> th;
  for (size_t t = 1; t < nthreads; t++) th.emplace_back(work, t);
  work(0);
  for (auto &t : th) t.join();
  bool ok = true;
  for (const auto &s : parts) ok = ok && std::fwrite(s.data(), 1, s.size(), f) == s.size();
  return ok && std::fputc('\n', f) != EOF;
}

}  // namespace

extern "C" omc_status omc_write_3ddose(const char *path, const omc_phantom *ph, const double *dose,
                                       const double *unc) {
  if (!path || !ph || !dose || !unc) return fail(OMC_ERR_ARG, "null argument");
  FILE *f = std::fopen(path, "w");
  if (!f) return fail(OMC_ERR_IO, "Unable to open file: %s", path);
  int nx = ph->nx, ny = ph->ny, nz = ph->nz;
  std::fprintf(f, "%5d%5d%5d\n", nx, ny, nz);
  for (int i = 0; i <= nx; i++) std::fprintf(f, "%f ", ph->xbounds[i]);
  std::fprintf(f, "\n");
  for (int i = 0; i <= ny; i++) std::fprintf(f, "%f ", ph->ybounds[i]);
  std::fprintf(f, "\n");
  for (int i = 0; i <= nz; i++) std::fprintf(f, "%f ", ph->zbounds[i]);
  std::fprintf(f, "\n");
  size_t nv = static_cast<size_t>(nx) * ny * nz;
  // Both arrays are formatted in parallel chunks and written in order.
  // std::to_chars with a precision produces the text printf produces for
  // "%.6e" / "%.6f" in the C locale, so the file is the reference's byte
  // for byte.
  bool ok = write_formatted(f, dose + 1, nv, std::chars_format::scientific) &&
            write_formatted(f, unc + 1, nv, std::chars_format::fixed);
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) return fail(OMC_ERR_IO, "writing %s failed", path);
  return OMC_OK;
}
