// Dose server: continuous batching of dose jobs on one GPU (omc_server_*).
//
// Two threads share one engine (tables resident once):
//  - admission: takes queued jobs in arrival order, maps their media onto
//    the server's media, builds their regions (initRegions semantics) and
//    uploads them (omc_engine_job_add, or omc_engine_job_add_dij for
//    beamlet jobs) while rounds run on the engine's compute stream, as far
//    as the device-memory budget and the job limit allow;
//  - scheduler: runs rounds over the resident jobs, field and beamlet
//    jobs together (omc_engine_job_round, one launch), reads back and frees
//    the jobs that finished (a beamlet job as its CSC dij), and wakes their
//    waiters and the admission thread.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "common.h"

using omc::fail;

namespace {

using Clock = std::chrono::steady_clock;

struct PhantomCopy {
  int nx = 0, ny = 0, nz = 0;
  std::vector<double> xb, yb, zb, density;
  std::vector<int> med;  // indices into the server's media (1-based, 0 vacuum)
};

enum class JobState { Queued, Resident, Done, Failed };

struct Job {
  long long id = 0;
  PhantomCopy ph;
  omc_source src{};
  double ecut = 0, pcut = 0;
  long long nperbatch = 0;
  int nbatch = 0;
  size_t bytes = 0;
  JobState state = JobState::Queued;
  omc_job *dev = nullptr;
  std::vector<double> acc, acc2;
  double ensrc = 0;
  double submit_s = 0, admit_s = 0, finish_s = 0;
  int rounds = 0;
  omc_status status = OMC_OK;
  // beamlet (dij) jobs: resident like field jobs, converted to CSC when done
  bool dij = false;
  int nbeams = 0;
  std::vector<int> ibeam;
  std::vector<double> bl[12];  // x/y/z source (nbeams), corner, side1, side2 (nbeamlets)
  std::vector<long long> nhist;
  double rel_threshold = 0;
  int fp32_values = 0;
  omc_dij *dij_out = nullptr;
  long long total() const {
    long long t = 0;
    for (long long h : nhist) t += h;
    return t;
  }
};

}  // namespace

struct omc_server {
  omc_server_config cfg{};
  omc_engine *eng = nullptr;
  omc_tables *tab = nullptr;
  std::vector<std::string> media;
  Clock::time_point t0;
  std::mutex mu;
  std::condition_variable cv_admit, cv_sched, cv_done;
  std::deque<std::shared_ptr<Job>> queued;
  std::vector<std::shared_ptr<Job>> resident;
  std::map<long long, std::shared_ptr<Job>> jobs;
  long long next_id = 1;
  long long resident_bytes = 0;
  bool stop = false;
  bool adaptive_rounds = false;  // round_histories chosen per round
  omc_server_stats st{};
  std::thread admit_thread, sched_thread;

  double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

// Round size bounds of the adaptive rounds (round_histories = 0).
constexpr long long kRoundMin = 4000000;
constexpr long long kRoundMax = 32000000;
constexpr size_t kFewJobs = 2;

// A job's phantom with its media renumbered onto the server's, and its
// regions against the server's tables (initRegions, omc_regions_build).
struct JobGeometry {
  omc_phantom *ph = nullptr;
  omc_input *in = nullptr;
  omc_regions *reg = nullptr;
  ~JobGeometry() {
    omc_regions_free(reg);
    omc_input_free(in);
    omc_phantom_free(ph);
  }
};

omc_status job_geometry(omc_server *s, const Job &j, JobGeometry &g) {
  omc_status st;
  std::vector<const char *> names;
  for (const auto &m : s->media) names.push_back(m.c_str());
  if ((st = omc_phantom_create(static_cast<int>(names.size()), names.data(), j.ph.nx, j.ph.ny, j.ph.nz,
                               j.ph.xb.data(), j.ph.yb.data(), j.ph.zb.data(), j.ph.med.data(), j.ph.density.data(),
                               &g.ph)) != OMC_OK)
    return st;
  char text[256];
  std::snprintf(text, sizeof text, "global ecut = %.17g\nglobal pcut = %.17g\n", j.ecut, j.pcut);
  if ((st = omc_input_from_string(text, &g.in)) != OMC_OK) return st;
  return omc_regions_build(g.in, g.ph, s->tab, &g.reg);
}

// A job goes onto the device at admission: phantom, source, tallies (and
// beamlets).
omc_status upload_job(omc_server *s, Job &j) {
  JobGeometry g;
  omc_status st = job_geometry(s, j, g);
  if (st != OMC_OK) return st;
  if (!j.dij)
    return omc_engine_job_add(s->eng, g.ph, g.reg, &j.src, j.nperbatch, j.nbatch, s->cfg.precision, &j.dev);
  omc_beamlets b{static_cast<int>(j.ibeam.size()), j.nbeams, j.ibeam.data(), j.bl[0].data(), j.bl[1].data(),
                 j.bl[2].data(), j.bl[3].data(), j.bl[4].data(), j.bl[5].data(), j.bl[6].data(), j.bl[7].data(),
                 j.bl[8].data(), j.bl[9].data(), j.bl[10].data(), j.bl[11].data()};
  return omc_engine_job_add_dij(s->eng, g.ph, g.reg, &j.src, &b, j.nhist.data(), 0, j.nbatch, s->cfg.precision,
                                &j.dev);
}

void admission_loop(omc_server *s) {
  std::unique_lock<std::mutex> lk(s->mu);
  for (;;) {
    s->cv_admit.wait(lk, [&] {
      if (s->stop) return true;
      if (s->queued.empty()) return false;
      const auto &h = s->queued.front();
      bool fits = s->resident_bytes + static_cast<long long>(h->bytes) <= s->cfg.hbm_budget ||
                  s->resident.empty();  // a job larger than the budget still runs, alone
      return fits && static_cast<int>(s->resident.size()) < s->cfg.max_jobs;
    });
    if (s->stop) return;
    std::shared_ptr<Job> j = s->queued.front();
    s->queued.pop_front();
    s->resident_bytes += static_cast<long long>(j->bytes);
    lk.unlock();
    omc_status st = upload_job(s, *j);
    lk.lock();
    if (st != OMC_OK) {
      s->resident_bytes -= static_cast<long long>(j->bytes);
      j->status = st;
      j->state = JobState::Failed;
      j->finish_s = s->now();
      s->cv_done.notify_all();
      continue;
    }
    j->admit_s = s->now();
    j->state = JobState::Resident;
    s->resident.push_back(j);
    s->st.max_resident = std::max(s->st.max_resident, static_cast<int>(s->resident.size()));
    s->st.max_resident_bytes = std::max(s->st.max_resident_bytes, s->resident_bytes);
    s->cv_sched.notify_all();
  }
}

void scheduler_loop(omc_server *s) {
  // The lanes' RANMAR streams are seeded once and continue from round to
  // round, so no number is drawn twice.
  bool seeded = false;
  std::unique_lock<std::mutex> lk(s->mu);
  for (;;) {
    s->cv_sched.wait(lk, [&] { return s->stop || !s->resident.empty(); });
    if (s->stop) return;
    std::vector<std::shared_ptr<Job>> all = s->resident;
    lk.unlock();
    std::vector<std::shared_ptr<Job>> round = all;  // field and beamlet jobs alike
    std::vector<long long> left(round.size()), quota(round.size(), 0);
    long long backlog = 0, shortest = -1;
    for (size_t i = 0; i < round.size(); i++) {
      left[i] = omc_job_histories(round[i]->dev) - omc_job_done(round[i]->dev);
      backlog += left[i];
      if (left[i] > 0 && (shortest < 0 || left[i] < shortest)) shortest = left[i];
    }
    const long long R = omc_server_round_histories(s->adaptive_rounds ? 0 : s->cfg.round_histories, backlog,
                                                   shortest, static_cast<int>(round.size()));
    long long budget = R;
    if (s->cfg.policy == OMC_SERVE_EQUAL_SHARES) {
      // Equal shares; a job with fewer histories left takes only those and
      // its unused share goes to the others.
      size_t open = round.size();
      while (budget > 0 && open > 0) {
        long long share = std::max<long long>(1, budget / static_cast<long long>(open));
        open = 0;
        for (size_t i = 0; i < round.size(); i++) {
          long long take = std::min(share, left[i] - quota[i]);
          if (take <= 0) continue;
          if (take > budget) take = budget;
          quota[i] += take;
          budget -= take;
          if (left[i] - quota[i] > 0) open++;
        }
      }
    } else {
      // Shortest remaining first: the round is filled with the jobs that
      // have the fewest histories left (arrival order among equals), so
      // small jobs finish in the next round and large ones take the rest.
      std::vector<size_t> order(round.size());
      for (size_t i = 0; i < order.size(); i++) order[i] = i;
      std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return left[a] < left[b]; });
      for (size_t i : order) {
        if (budget <= 0) break;
        quota[i] = std::min(left[i], budget);
        budget -= quota[i];
      }
    }
    std::vector<omc_job *> devs;
    std::vector<long long> q;
    std::vector<std::shared_ptr<Job>> in_round;
    for (size_t i = 0; i < round.size(); i++)
      if (quota[i] > 0) {
        devs.push_back(round[i]->dev);
        q.push_back(quota[i]);
        in_round.push_back(round[i]);
      }
    omc_status st = OMC_OK;
    omc_run_stats rs{};
    if (!devs.empty()) {
      omc_run_config rc;
      std::memset(&rc, 0, sizeof rc);
      rc.nbatch = 1;
      rc.ixx = s->cfg.ixx;
      rc.jxx = s->cfg.jxx;
      rc.nsplit = s->cfg.nsplit;
      rc.precision = s->cfg.precision;
      rc.continue_streams = seeded ? 1 : 0;
      st = omc_engine_job_round(s->eng, devs.data(), q.data(), static_cast<int>(devs.size()), &rc, &rs);
      seeded = true;
    }
    // Jobs that are complete (or hit by a failed round) leave the device.
    std::vector<std::shared_ptr<Job>> finished;
    for (auto &j : in_round) {
      j->rounds++;
      bool failed_round = st != OMC_OK;
      if (failed_round || omc_job_done(j->dev) >= omc_job_histories(j->dev)) {
        if (!failed_round && j->dij) {
          j->status = omc_engine_job_dij(s->eng, j->dev, j->rel_threshold, j->fp32_values, &j->dij_out);
        } else if (!failed_round) {
          j->acc.assign(j->ph.nx * static_cast<size_t>(j->ph.ny) * j->ph.nz + 1, 0.0);
          j->acc2.assign(j->acc.size(), 0.0);
          j->status = omc_engine_job_result(s->eng, j->dev, j->acc.data(), j->acc2.data(), &j->ensrc);
        } else {
          j->status = st;
        }
        omc_engine_job_remove(s->eng, j->dev);
        j->dev = nullptr;
        finished.push_back(j);
      }
    }
    lk.lock();
    s->st.rounds++;
    s->st.histories += rs.histories;
    s->st.transport_s += rs.transport_ms * 1e-3;
    s->st.max_round_jobs = std::max(s->st.max_round_jobs, static_cast<int>(devs.size()));
    for (auto &j : finished) {
      j->finish_s = s->now();
      j->state = j->status == OMC_OK ? JobState::Done : JobState::Failed;
      s->resident.erase(std::remove(s->resident.begin(), s->resident.end(), j), s->resident.end());
      s->resident_bytes -= static_cast<long long>(j->bytes);
      s->st.finished++;
    }
    if (!finished.empty()) {
      s->cv_done.notify_all();
      s->cv_admit.notify_all();
    }
  }
}

}  // namespace

// A round ends with a tail in which its last histories finish at low
// occupancy (about 40 ms on a GB300, whatever the round's size), so short
// rounds cost throughput and long ones make arrivals and small jobs wait.
// While few jobs are resident (a lightly loaded server) a round takes a
// quarter of the backlog, but at most four times the histories the
// shortest job has left, between kRoundMin and kRoundMax; with more jobs
// resident, kRoundMin, so that the small ones among them and new arrivals
// pass the large ones soon.
extern "C" long long omc_server_round_histories(long long configured, long long backlog, long long shortest,
                                                int resident) {
  if (configured > 0) return configured;
  if (resident > static_cast<int>(kFewJobs)) return kRoundMin;
  const long long r = std::min(backlog / 4, 4 * std::max(shortest, 0ll));
  return std::min(kRoundMax, std::max(kRoundMin, r));
}

extern "C" omc_status omc_server_create(const omc_server_config *cfg, const omc_input *data_keys, int nmed,
                                        const char *const *media, omc_server **out) {
  if (!cfg || !data_keys || !media || !out) return fail(OMC_ERR_ARG, "null argument");
  *out = nullptr;
  if (nmed < 1 || nmed > OMC_MXMED) return fail(OMC_ERR_ARG, "between 1 and %d media", OMC_MXMED);
  if (cfg->precision != OMC_FP32 && cfg->precision != OMC_FP64) return fail(OMC_ERR_ARG, "unknown precision");
  std::unique_ptr<omc_server> s(new omc_server());
  s->cfg = *cfg;
  if (s->cfg.max_jobs <= 0) s->cfg.max_jobs = 256;
  s->adaptive_rounds = s->cfg.round_histories <= 0;
  if (s->cfg.nsplit <= 0) s->cfg.nsplit = 1;
  char names[OMC_MXMED][OMC_NAME_LEN];
  std::memset(names, 0, sizeof names);
  for (int i = 0; i < nmed; i++) {
    if (!media[i] || std::strlen(media[i]) >= OMC_NAME_LEN) return fail(OMC_ERR_ARG, "medium name %d", i);
    std::strcpy(names[i], media[i]);
    s->media.emplace_back(media[i]);
  }
  omc_status st;
  if ((st = omc_tables_build(data_keys, nmed, names, &s->tab)) != OMC_OK) return st;
  if ((st = omc_engine_create(cfg->device, &s->eng)) != OMC_OK) {
    omc_tables_free(s->tab);
    return st;
  }
  if ((st = omc_engine_set_tables(s->eng, s->tab)) != OMC_OK) {
    omc_engine_destroy(s->eng);
    omc_tables_free(s->tab);
    return st;
  }
  if (s->cfg.hbm_budget <= 0) {
    size_t fr = 0, tot = 0;
    omc_device_memory(cfg->device, &fr, &tot);
    s->cfg.hbm_budget = static_cast<long long>(fr / 2);
  }
  s->t0 = Clock::now();
  omc_server *raw = s.get();
  s->admit_thread = std::thread(admission_loop, raw);
  s->sched_thread = std::thread(scheduler_loop, raw);
  *out = s.release();
  return OMC_OK;
}

namespace {

// Host copy of a job, its media renumbered onto the server's by name.
omc_status copy_job(omc_server *s, const omc_server_job *job, std::shared_ptr<Job> &out) {
  const omc_phantom *p = job->phantom;
  auto j = std::make_shared<Job>();
  j->ph.nx = p->nx;
  j->ph.ny = p->ny;
  j->ph.nz = p->nz;
  size_t nv = static_cast<size_t>(p->nx) * p->ny * p->nz;
  j->ph.xb.assign(p->xbounds, p->xbounds + p->nx + 1);
  j->ph.yb.assign(p->ybounds, p->ybounds + p->ny + 1);
  j->ph.zb.assign(p->zbounds, p->zbounds + p->nz + 1);
  j->ph.density.assign(p->density, p->density + nv);
  // Media onto the server's list by name.
  std::vector<int> map(p->nmed + 1, 0);
  for (int m = 0; m < p->nmed; m++) {
    auto it = std::find(s->media.begin(), s->media.end(), std::string(p->med_names[m]));
    if (it == s->media.end()) return fail(OMC_ERR_MEDIA, "medium %s is not one of the server's", p->med_names[m]);
    map[m + 1] = static_cast<int>(it - s->media.begin()) + 1;
  }
  j->ph.med.resize(nv);
  for (size_t v = 0; v < nv; v++) {
    int m = p->med_index[v];
    if (m < 0 || m > p->nmed) return fail(OMC_ERR_ARG, "voxel %zu: medium %d outside 0..%d", v, m, p->nmed);
    j->ph.med[v] = map[m];
  }
  j->src = *job->source;
  j->ecut = job->ecut;
  j->pcut = job->pcut;
  j->nperbatch = job->nperbatch;
  j->nbatch = job->nbatch;
  out = j;
  return OMC_OK;
}

void enqueue(omc_server *s, const std::shared_ptr<Job> &j, long long *id) {
  std::lock_guard<std::mutex> lk(s->mu);
  j->id = s->next_id++;
  j->submit_s = s->now();
  s->jobs[j->id] = j;
  s->queued.push_back(j);
  s->st.submitted++;
  *id = j->id;
  s->cv_admit.notify_all();
}

}  // namespace

extern "C" omc_status omc_server_submit(omc_server *s, const omc_server_job *job, long long *id) {
  if (!s || !job || !job->phantom || !job->source || !id) return fail(OMC_ERR_ARG, "null argument");
  if (job->nbatch < 1 || job->nperbatch < 1) return fail(OMC_ERR_ARG, "need nbatch >= 1 and nperbatch >= 1");
  std::shared_ptr<Job> j;
  omc_status st = copy_job(s, job, j);
  if (st != OMC_OK) return st;
  j->bytes = omc_job_device_bytes(job->phantom, job->nbatch, s->cfg.precision);
  enqueue(s, j, id);
  return OMC_OK;
}

extern "C" omc_status omc_server_submit_dij(omc_server *s, const omc_server_job *job, const omc_beamlets *bl,
                                            const long long *nhist, double rel_threshold, int fp32_values,
                                            long long *id) {
  if (!s || !job || !job->phantom || !job->source || !bl || !id) return fail(OMC_ERR_ARG, "null argument");
  if (job->nbatch < 1) return fail(OMC_ERR_ARG, "need nbatch >= 1");
  if (bl->nbeamlets < 1 || bl->nbeams < 1) return fail(OMC_ERR_ARG, "need at least one beamlet and one beam");
  if (bl->nbeamlets > 4096) return fail(OMC_ERR_ARG, "at most 4096 beamlets per job");
  if (!(rel_threshold >= 0.0)) return fail(OMC_ERR_ARG, "relative dose threshold must be >= 0");
  for (int i = 0; i < bl->nbeamlets; i++)
    if (bl->ibeam[i] < 0 || bl->ibeam[i] >= bl->nbeams) return fail(OMC_ERR_ARG, "beamlet %d: bad beam", i);
  if (nhist)
    for (int i = 0; i < bl->nbeamlets; i++)
      if (nhist[i] < 1) return fail(OMC_ERR_ARG, "beamlet %d: need at least one history", i);
  if (!nhist && job->nperbatch < 1) return fail(OMC_ERR_ARG, "need nperbatch >= 1");
  std::shared_ptr<Job> j;
  omc_status st = copy_job(s, job, j);
  if (st != OMC_OK) return st;
  j->dij = true;
  j->nbeams = bl->nbeams;
  j->ibeam.assign(bl->ibeam, bl->ibeam + bl->nbeamlets);
  const double *src[12] = {bl->xsource, bl->ysource, bl->zsource, bl->xcorner, bl->ycorner, bl->zcorner,
                           bl->xside1,  bl->yside1,  bl->zside1,  bl->xside2,  bl->yside2,  bl->zside2};
  for (int k = 0; k < 12; k++) j->bl[k].assign(src[k], src[k] + (k < 3 ? bl->nbeams : bl->nbeamlets));
  j->nhist.resize(bl->nbeamlets);
  for (int i = 0; i < bl->nbeamlets; i++)
    j->nhist[i] = nhist ? nhist[i] : job->nperbatch * static_cast<long long>(job->nbatch);
  j->rel_threshold = rel_threshold;
  j->fp32_values = fp32_values;
  // Device footprint while resident: phantom, source, beamlets and one
  // tally per beamlet.
  j->bytes = omc_job_dij_device_bytes(job->phantom, bl->nbeamlets, s->cfg.precision);
  enqueue(s, j, id);
  return OMC_OK;
}

extern "C" omc_status omc_server_wait_dij(omc_server *s, long long id, double timeout_s, omc_dij **out,
                                         omc_server_result *res) {
  if (!s || !out) return fail(OMC_ERR_ARG, "null argument");
  *out = nullptr;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->jobs.find(id);
  if (it == s->jobs.end()) return fail(OMC_ERR_ARG, "unknown job %lld", id);
  std::shared_ptr<Job> j = it->second;
  if (!j->dij) return fail(OMC_ERR_ARG, "job %lld is not a beamlet job", id);
  auto done = [&] { return j->state == JobState::Done || j->state == JobState::Failed; };
  if (timeout_s < 0) {
    s->cv_done.wait(lk, done);
  } else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), done)) {
    return fail(OMC_ERR_LIMIT, "job %lld not finished after %.3f s", id, timeout_s);
  }
  s->jobs.erase(it);
  if (res) {
    res->ensrc = 0;
    res->histories = j->total();
    res->submit_s = j->submit_s;
    res->admit_s = j->admit_s;
    res->finish_s = j->finish_s;
    res->rounds = j->rounds;
    res->status = j->status;
  }
  if (j->state == JobState::Failed) return fail(j->status, "job %lld failed", id);
  *out = j->dij_out;
  j->dij_out = nullptr;
  return OMC_OK;
}

extern "C" omc_status omc_server_wait(omc_server *s, long long id, double timeout_s, double *accum_endep,
                                      double *accum_endep2, omc_server_result *res) {
  if (!s) return fail(OMC_ERR_ARG, "null argument");
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->jobs.find(id);
  if (it == s->jobs.end()) return fail(OMC_ERR_ARG, "unknown job %lld", id);
  std::shared_ptr<Job> j = it->second;
  if (j->dij) return fail(OMC_ERR_ARG, "job %lld is a beamlet job: use omc_server_wait_dij", id);
  auto done = [&] { return j->state == JobState::Done || j->state == JobState::Failed; };
  if (timeout_s < 0) {
    s->cv_done.wait(lk, done);
  } else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), done)) {
    return fail(OMC_ERR_LIMIT, "job %lld not finished after %.3f s", id, timeout_s);
  }
  s->jobs.erase(it);
  if (res) {
    res->ensrc = j->ensrc;
    res->histories = j->nperbatch * j->nbatch;
    res->submit_s = j->submit_s;
    res->admit_s = j->admit_s;
    res->finish_s = j->finish_s;
    res->rounds = j->rounds;
    res->status = j->status;
  }
  if (j->state == JobState::Failed) return fail(j->status, "job %lld failed", id);
  if (accum_endep) std::copy(j->acc.begin(), j->acc.end(), accum_endep);
  if (accum_endep2) std::copy(j->acc2.begin(), j->acc2.end(), accum_endep2);
  return OMC_OK;
}

extern "C" omc_status omc_server_get_stats(omc_server *s, omc_server_stats *st) {
  if (!s || !st) return fail(OMC_ERR_ARG, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  *st = s->st;
  return OMC_OK;
}

extern "C" void omc_server_destroy(omc_server *s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_admit.notify_all();
  s->cv_sched.notify_all();
  if (s->admit_thread.joinable()) s->admit_thread.join();
  if (s->sched_thread.joinable()) s->sched_thread.join();
  for (auto &j : s->resident)
    if (j->dev) omc_engine_job_remove(s->eng, j->dev);
  s->resident.clear();
  for (auto &kv : s->jobs)
    if (kv.second->dij_out) omc_dij_free(kv.second->dij_out);
  omc_engine_destroy(s->eng);
  omc_tables_free(s->tab);
  delete s;
}
