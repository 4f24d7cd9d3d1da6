// matRad entry point: the omc_matrad front end's mexFunction
// (ucodes/omc_matrad/omc_matrad.c:1258-1530) as a C function over plain
// arrays.  parseInput (:62-250) becomes .inp text for the host library,
// initPhantom (:269-342) a phantom over the caller's cube, and the beamlet
// loop one omc_engine_run_dij call.
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>

#include "common.h"

using omc::fail;

namespace {

std::string num(double v) {
  char b[64];
  std::snprintf(b, sizeof b, "%.17g", v);
  return b;
}

struct Cleanup {
  omc_input *in = nullptr;
  omc_phantom *ph = nullptr;
  omc_tables *tab = nullptr;
  omc_regions *reg = nullptr;
  omc_source *src = nullptr;
  omc_engine *eng = nullptr;
  ~Cleanup() {
    omc_engine_destroy(eng);
    omc_source_free(src);
    omc_regions_free(reg);
    omc_tables_free(tab);
    omc_phantom_free(ph);
    omc_input_free(in);
  }
};

}  // namespace

extern "C" omc_status omc_matrad_dij(int device, const omc_matrad_geo *geo, const omc_beamlets *bl,
                                     const omc_matrad_opt *opt, int precision, int serial, omc_dij **out) {
  if (!geo || !bl || !opt || !out) return fail(OMC_ERR_ARG, "null argument");
  *out = nullptr;
  if (!geo->cube_rho || !geo->cube_mat_ix || !geo->materials || !geo->xbounds || !geo->ybounds || !geo->zbounds)
    return fail(OMC_ERR_ARG, "null geometry array");
  if (!opt->pegs_file || !opt->pgs4form_file || !opt->data_folder)
    return fail(OMC_ERR_ARG, "pegsFile, pgs4formFile and dataFolder are required");
  if (opt->n_batches < 1) return fail(OMC_ERR_ARG, "nBatches must be >= 1");
  // parseInput: the mcOpt fields as input keys.  The reference's source
  // reads neither collimator nor SSD and never sets the charge (beams are
  // photons); the host source builder gets neutral values for those keys.
  std::string text;
  text += "ncase = " + std::to_string(opt->n_histories) + "\n";
  text += "nbatch = " + std::to_string(opt->n_batches) + "\n";
  text += "nsplit = " + std::to_string(opt->n_split) + "\n";
  if (opt->spectrum_file && opt->spectrum_file[0]) text += std::string("spectrum file = ") + opt->spectrum_file + "\n";
  text += "mono energy = " + num(opt->mono_energy) + "\n";
  text += "charge = 0\ncollimator bounds = 0 0 0 0\nssd = 100\n";
  text += "global ecut = " + num(opt->global_ecut) + "\n";
  text += "global pcut = " + num(opt->global_pcut) + "\n";
  text += "rng seeds = " + std::to_string(opt->random_seeds[0]) + " " + std::to_string(opt->random_seeds[1]) + "\n";
  text += std::string("pegs file = ") + opt->pegs_file + "\n";
  text += std::string("pgs4form file = ") + opt->pgs4form_file + "\n";
  text += std::string("data folder = ") + opt->data_folder + "\n";
  text += std::string("output folder = ") + (opt->output_folder ? opt->output_folder : "") + "\n";
  Cleanup c;
  omc_status s;
  if ((s = omc_input_from_string(text.c_str(), &c.in)) != OMC_OK) return s;
  if ((s = omc_phantom_create(geo->nmaterials, geo->materials, geo->nx, geo->ny, geo->nz, geo->xbounds, geo->ybounds,
                              geo->zbounds, geo->cube_mat_ix, geo->cube_rho, &c.ph)) != OMC_OK)
    return s;
  if ((s = omc_tables_build(c.in, c.ph->nmed, static_cast<const char(*)[OMC_NAME_LEN]>(c.ph->med_names), &c.tab)) !=
      OMC_OK)
    return s;
  if ((s = omc_source_build(c.in, c.ph, &c.src)) != OMC_OK) return s;
  if ((s = omc_regions_build(c.in, c.ph, c.tab, &c.reg)) != OMC_OK) return s;
  if ((s = omc_engine_create(device, &c.eng)) != OMC_OK) return s;
  if ((s = omc_engine_set_tables(c.eng, c.tab)) != OMC_OK) return s;
  if ((s = omc_engine_set_geometry(c.eng, c.ph, c.reg)) != OMC_OK) return s;
  if ((s = omc_engine_set_source(c.eng, c.src)) != OMC_OK) return s;
  if ((s = omc_engine_set_beamlets(c.eng, bl)) != OMC_OK) return s;
  // Histories per beamlet as the reference counts them (omc_matrad.c:
  // 1321-1335): nhist/nbatch per batch, at least one.
  long long nhist = opt->n_histories;
  if (nhist / opt->n_batches == 0) nhist = opt->n_batches;
  omc_run_config cfg;
  std::memset(&cfg, 0, sizeof cfg);
  cfg.nperbatch = nhist / opt->n_batches;
  cfg.nbatch = opt->n_batches;
  cfg.ixx = opt->random_seeds[0];
  cfg.jxx = opt->random_seeds[1];
  cfg.nsplit = opt->n_split;
  cfg.precision = precision;
  cfg.serial = serial;
  omc_dij_config dc;
  std::memset(&dc, 0, sizeof dc);
  dc.rel_threshold = opt->rel_dose_threshold;
  omc_run_stats st;
  std::memset(&st, 0, sizeof st);
  if (opt->verbose)
    std::printf("omc_matrad: %d beamlets, %lld histories each in %d batches, relative dose cut-off %f\n",
                bl->nbeamlets, cfg.nperbatch * cfg.nbatch, cfg.nbatch, dc.rel_threshold);
  s = omc_engine_run_dij(c.eng, &cfg, &dc, out, &st);
  if (opt->verbose && *out)
    std::printf("Sparse MC Dij has %lld (%f percent) elements! Transport %.3f s on the GPU\n", (*out)->nnz,
                100.0 * static_cast<double>((*out)->nnz) /
                    (static_cast<double>((*out)->nrows) * static_cast<double>((*out)->ncols)),
                st.transport_ms * 1e-3);
  return s;
}
