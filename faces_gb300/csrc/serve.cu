// serve.cu -- a job server: halo-sum jobs of different sizes arrive over
// time; each is admitted against an HBM budget, keeps its field resident on
// the device for all its shares, and every share of every running job
// happens in one persistent launch per tick (continuous batching).
//
// Scheduling, on the host thread that calls faces_server_poll:
//   retire -- ticks whose completion event has fired: their finishing jobs
//             become done, with the GPU completion time of that tick;
//   admit  -- queued jobs in arrival order while the budget and the job
//             limit allow (a job that does not fit holds the ones behind it,
//             so a large job is never starved): the field comes from a
//             stream-ordered pool and is initialised on the device;
//   launch -- one share of every running job in one launch of the batched
//             tile kernel (batch_kernel.h) over a work list rebuilt only when
//             the set of running jobs changes.  Up to kDepth ticks are in
//             flight, so the host prepares the next while the GPU runs one.
// Everything is enqueued on one stream, so a job admitted during a tick
// starts at the next one and its memory is reused only after its last tick.
// Completion times come from CUDA events measured against a base event whose
// host time is known, so latencies are GPU completion minus arrival.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <new>
#include <thread>
#include <tuple>
#include <vector>

#include "../../include/faces_gb300.h"
#include "batch_kernel.h"
#include "geom.cuh"
#include "kernels.cuh"
#include "rows_setup.cuh"
#include "ptile_steps.cuh"
#include "tables.h"

void faces_internal_set_error(const char *msg);

using namespace faces;

namespace {

int fail(int code, const char *fmt, ...)
{
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  faces_internal_set_error(buf);
  return code;
}

#define CUDA_TRY(call, what)                                                                      \
  do {                                                                                            \
    cudaError_t e_ = (call);                                                                      \
    if (e_ != cudaSuccess)                                                                        \
      return fail(e_ == cudaErrorMemoryAllocation ? FACES_ENOMEM : FACES_ECUDA, "%s: %s", what, \
                  cudaGetErrorString(e_));                                                        \
  } while (0)

constexpr int kDepth = 2;  // ticks in flight
// work units of whole columns, one per block in a row (see launch_batch):
// the fastest of the settings timed on the served workload (1.56x the plain
// form saturated; one-chunk units and runs of 8 gave 1.43-1.44x)
constexpr int kServeUnitDiv = 1;
constexpr int kServeRun = 1;

enum JobState { kQueued = 0, kRunning = 1, kDone = 2, kReleased = 3 };

struct Job {
  long long id = 0;
  faces_job spec{};
  FieldDesc f{};
  RowPlan tp{};    // single-field tile plan (plain form)
  long tgrid = 0;  // single-field tile kernel blocks (plain form)
  size_t bytes = 0;
  int shares_left = 0, shares_done = 0;
  int state = kQueued;
  double t_submit = 0, t_admit = 0, t_done = 0;  // server clock, seconds
};

struct Tick {
  cudaEvent_t ev = nullptr;
  std::vector<long long> finishing;  // jobs whose last share is in this tick
  char *staging = nullptr;           // pinned copy source of the work list
  size_t staging_cap = 0;
};

double host_seconds()
{
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

}  // namespace

struct faces_server {
  size_t budget = 0, resident = 0, peak_resident = 0;
  int max_jobs = 0;
  unsigned flags = 0;
  int sms = 0;
  cudaStream_t stream = nullptr, fetch_stream = nullptr;
  cudaMemPool_t pool = nullptr;
  cudaEvent_t base = nullptr;
  double base_host = 0;  // host clock at the base event
  long long next_id = 1;
  std::map<long long, Job> jobs;
  std::deque<long long> queue;
  std::vector<long long> running;  // admitted, shares left
  bool set_changed = true;
  // device work list of the current running set (pool memory): the field
  // table, then the units from tables_fbytes on
  char *d_tables = nullptr;
  size_t tables_fbytes = 0;
  int nunits = 0;
  int kmode = 0, khalf = 0;  // kernel form of the running set's work list
  int unit_div = kServeUnitDiv, run = kServeRun, half = 0;  // work list settings (faces_server_tune)
  int warp_n = kBatchWarpMaxN, boost = 2;  // the warp form (faces_server_tune_warp)
  int nsmall = 0, wblocks = 0;
  long grid = 0;
  Tick ticks[kDepth];
  int tick_head = 0, in_flight = 0;  // ring of in-flight ticks
  std::map<std::tuple<int, int, int, int>, std::pair<int *, std::vector<int>>> nbr_cache;
  // counters
  long long submitted = 0, admitted = 0, completed = 0, nticks = 0, job_shares = 0, launches = 0;
  double point_shares = 0;
};

namespace {

double gpu_time_of(faces_server *s, cudaEvent_t ev)
{
  float ms = 0;
  cudaEventElapsedTime(&ms, s->base, ev);
  return s->base_host + ms * 1e-3;
}

int validate(const faces_server *s, const faces_job *j, size_t *bytes)
{
  if (!j) return fail(FACES_EINVAL, "null job");
  if (j->lx < 1 || j->ly < 1 || j->lz < 1 || j->mx < 1 || j->my < 1 || j->mz < 1)
    return fail(FACES_EINVAL, "job: rank grid and element grid must be positive");
  if (!batch_n_supported(j->n))
    return fail(FACES_EUNSUPPORTED, "job: n = %d; the server runs %d <= n <= %d", j->n, kBatchMinN, kBatchMaxN);
  if (j->flags & ~FACES_PERIODIC)
    return fail(FACES_EUNSUPPORTED, "job: flags 0x%x; the server runs direct mode (FACES_PERIODIC or 0)", j->flags);
  if (j->nshares < 1) return fail(FACES_EINVAL, "job: nshares = %d must be at least 1", j->nshares);
  if (j->init < 0 || j->init > 2 || (j->init == 2 && !j->host_in))
    return fail(FACES_EINVAL, "job: init = %d (0 reference, 1 integer seed, 2 host data with host_in)", j->init);
  const long nranks = (long)j->lx * j->ly * j->lz;
  const long doubles = nranks * jz_stride(j->n, j->mx, j->my) * j->mz;
  *bytes = (size_t)doubles * sizeof(double);
  if (*bytes > s->budget)
    return fail(FACES_EINVAL, "job: field of %zu bytes exceeds the server budget of %zu bytes", *bytes, s->budget);
  return FACES_OK;
}

// neighbour table of a rank grid, uploaded once per (lx, ly, lz, periodic)
int nbr_table(faces_server *s, const faces_job &j, const int **out)
{
  const auto key = std::make_tuple(j.lx, j.ly, j.lz, (j.flags & FACES_PERIODIC) ? 1 : 0);
  auto it = s->nbr_cache.find(key);
  if (it == s->nbr_cache.end()) {
    const int L[3] = {j.lx, j.ly, j.lz};
    std::vector<int> t = neighbour_table(L, std::get<3>(key) != 0);
    int *d = nullptr;
    CUDA_TRY(cudaMallocFromPoolAsync(reinterpret_cast<void **>(&d), t.size() * sizeof(int), s->pool, s->stream),
             "server: neighbour table");
    it = s->nbr_cache.emplace(key, std::make_pair(d, std::move(t))).first;
    CUDA_TRY(cudaMemcpyAsync(d, it->second.second.data(), it->second.second.size() * sizeof(int),
                             cudaMemcpyHostToDevice, s->stream),
             "server: neighbour table upload");
  }
  *out = it->second.first;
  return FACES_OK;
}

// the single-field tile kernel's plan for the plain form (as faces_share)
void plain_plan(faces_server *s, Job &job)
{
  const int n = job.f.n;
  job.tp = make_row_plan(job.f, tile_default_chunk(n), 0);
  job.tp.order = 2;
  job.tp.unit_chunks = ptile_field(job.f) ? 1 : (job.tp.nchunks + 1) / 2;
  job.tgrid = (long)s->sms * tile_blocks_per_sm(n, job.tp.chunk, tile_form(job.f, false));
}

int admit(faces_server *s, Job &job)
{
  const faces_job &j = job.spec;
  const int *nbr = nullptr;
  if (int rc = nbr_table(s, j, &nbr)) return rc;
  double *u = nullptr;
  CUDA_TRY(cudaMallocFromPoolAsync(reinterpret_cast<void **>(&u), job.bytes, s->pool, s->stream), "server: field");
  FieldDesc &f = job.f;
  f.u = u;
  f.n = j.n;
  f.m[0] = j.mx; f.m[1] = j.my; f.m[2] = j.mz;
  f.L[0] = j.lx; f.L[1] = j.ly; f.L[2] = j.lz;
  f.periodic = (j.flags & FACES_PERIODIC) ? 1 : 0;
  f.mode = kDirect;
  f.nranks = j.lx * j.ly * j.lz;
  f.sjy = (long)j.n * j.n * j.n * j.mx;
  f.sjz = jz_stride(j.n, j.mx, j.my);
  f.R = f.sjz * j.mz;
  f.msg = nullptr;
  f.msg_off = nullptr;
  f.recv_off = nullptr;
  f.nbr = nbr;
  plain_plan(s, job);
  cudaError_t e;
  if (j.init == 0) e = launch_init_ref(f, s->stream);
  else if (j.init == 1) e = launch_init_int(f, j.seed, s->stream);
  else e = cudaMemcpyAsync(u, j.host_in, job.bytes, cudaMemcpyHostToDevice, s->stream);
  if (e != cudaSuccess) {
    cudaFreeAsync(u, s->stream);
    f.u = nullptr;
    return fail(FACES_ECUDA, "server: job initialisation: %s", cudaGetErrorString(e));
  }
  if (j.init != 2) s->launches++;
  job.spec.host_in = nullptr;  // read by the copy above; not kept
  job.state = kRunning;
  job.shares_left = j.nshares;
  job.t_admit = host_seconds();
  s->resident += job.bytes;
  s->peak_resident = std::max(s->peak_resident, s->resident);
  s->admitted++;
  s->running.push_back(job.id);
  s->set_changed = true;
  return FACES_OK;
}

int release_job(faces_server *s, Job &job)
{
  if (job.f.u) {
    CUDA_TRY(cudaFreeAsync(job.f.u, s->stream), "server: free field");
    job.f.u = nullptr;
    s->resident -= job.bytes;
  }
  job.state = kReleased;
  return FACES_OK;
}

// retire completed ticks in order; wait: block on the oldest one
int retire(faces_server *s, bool wait, int *ndone)
{
  while (s->in_flight > 0) {
    Tick &t = s->ticks[s->tick_head];
    cudaError_t e = wait ? cudaEventSynchronize(t.ev) : cudaEventQuery(t.ev);
    if (e == cudaErrorNotReady) break;
    CUDA_TRY(e, "server: tick");
    const double tdone = gpu_time_of(s, t.ev);
    for (long long id : t.finishing) {
      Job &job = s->jobs[id];
      job.state = kDone;
      job.t_done = tdone;
      s->completed++;
      if (ndone) (*ndone)++;
      if (s->flags & FACES_SERVE_RELEASE_DONE)
        if (int rc = release_job(s, job)) return rc;
    }
    t.finishing.clear();
    s->tick_head = (s->tick_head + 1) % kDepth;
    s->in_flight--;
    wait = false;  // only the oldest
  }
  return FACES_OK;
}

int admit_queued(faces_server *s)
{
  while (!s->queue.empty()) {
    Job &job = s->jobs[s->queue.front()];
    if (s->resident + job.bytes > s->budget) break;
    if (s->max_jobs > 0 && (int)s->running.size() >= s->max_jobs) break;
    if (int rc = admit(s, job)) return rc;
    s->queue.pop_front();
  }
  return FACES_OK;
}

// work list of the running set, jobs in order of n: the field table then the
// units, staged in the tick's pinned buffer and copied to a pool allocation
int rebuild_tables(faces_server *s, Tick &t)
{
  std::vector<long long> order = s->running;
  std::stable_sort(order.begin(), order.end(),
                   [&](long long a, long long b) { return s->jobs[a].f.n < s->jobs[b].f.n; });
  // the kernel form: the tile form applies only when every job takes the
  // periodic step; plans are made for the form that runs
  int lean = 0;
  for (long long id : order) lean += ptile_field(s->jobs[id].f) ? 1 : 0;
  const int kmode = lean == 0 ? 0 : lean == (int)order.size() ? 1 : 2;
  const int half = kmode == 1 ? s->half : 0;
  std::vector<BatchField> fields;
  std::vector<BatchUnit> units;
  fields.reserve(order.size());
  // jobs of small n (the smallest, so listed first) take the warp form when
  // every job is on the periodic step
  int nsmall = 0;
  double small_pts = 0, large_pts = 0;
  for (long long id : order) {
    const Job &job = s->jobs[id];
    const bool warp = kmode == 1 && half != 1 && job.f.n <= s->warp_n && batch_warp_chunk(job.f.n) > 0;
    const RowPlan p = batch_plan(job.f, half, ptile_field(job.f), warp);
    append_units(units, (int)fields.size(), p, warp ? 1 : s->unit_div);
    fields.push_back({job.f, p, ptile_field(job.f) ? 1 : 0});
    const double pts = (double)job.f.nranks * job.f.m[0] * job.f.m[1] * job.f.m[2] * job.f.n * job.f.n * job.f.n;
    if (warp) {
      nsmall = (int)units.size();
      small_pts += pts;
    } else {
      large_pts += pts;
    }
  }
  int wblocks = 0;
  long grid = 0;
  warp_split((long)s->sms * batch_blocks_per_sm(half), nsmall, (long)units.size() - nsmall, small_pts, large_pts,
             s->boost, s->run, wblocks, grid);
  const size_t fbytes = (fields.size() * sizeof(BatchField) + 255) / 256 * 256;
  const size_t ubytes = units.size() * sizeof(BatchUnit);
  const size_t bytes = fbytes + ubytes;
  if (t.staging_cap < bytes) {
    // the tick is not in flight, so its last copy from the buffer is done
    if (t.staging) cudaFreeHost(t.staging);
    t.staging = nullptr;
    t.staging_cap = 0;
    CUDA_TRY(cudaHostAlloc(reinterpret_cast<void **>(&t.staging), bytes * 2, cudaHostAllocDefault),
             "server: pinned staging");
    t.staging_cap = bytes * 2;
  }
  std::memcpy(t.staging, fields.data(), fields.size() * sizeof(BatchField));
  std::memcpy(t.staging + fbytes, units.data(), ubytes);
  if (s->d_tables) CUDA_TRY(cudaFreeAsync(s->d_tables, s->stream), "server: free work list");
  s->d_tables = nullptr;
  CUDA_TRY(cudaMallocFromPoolAsync(reinterpret_cast<void **>(&s->d_tables), bytes, s->pool, s->stream),
           "server: work list");
  CUDA_TRY(cudaMemcpyAsync(s->d_tables, t.staging, bytes, cudaMemcpyHostToDevice, s->stream),
           "server: work list upload");
  s->tables_fbytes = fbytes;
  s->kmode = kmode;
  s->khalf = half;
  s->nunits = (int)units.size();
  s->nsmall = nsmall;
  s->wblocks = wblocks;
  s->grid = grid;
  s->set_changed = false;
  return FACES_OK;
}

// one share of every running job: one batched launch (or, in the plain
// form, one single-field launch per job), then the tick's event
int launch_tick(faces_server *s)
{
  Tick &t = s->ticks[(s->tick_head + s->in_flight) % kDepth];
  if (s->flags & FACES_SERVE_PLAIN) {
    for (long long id : s->running) {
      const Job &job = s->jobs[id];
      CUDA_TRY(launch_tiles(job.f, job.tp, job.tgrid, s->stream), "server: tile launch");
      s->launches++;
    }
  } else {
    if (s->set_changed)
      if (int rc = rebuild_tables(s, t)) return rc;
    CUDA_TRY(launch_batch(reinterpret_cast<const BatchField *>(s->d_tables),
                          reinterpret_cast<const BatchUnit *>(s->d_tables + s->tables_fbytes), s->nunits, s->grid,
                          s->run, s->kmode, s->khalf, s->stream, s->nsmall, s->wblocks),
             "server: batched launch");
    s->launches++;
  }
  CUDA_TRY(cudaEventRecord(t.ev, s->stream), "server: tick event");
  t.finishing.clear();
  std::vector<long long> still;
  still.reserve(s->running.size());
  for (long long id : s->running) {
    Job &job = s->jobs[id];
    job.shares_left--;
    job.shares_done++;
    s->job_shares++;
    s->point_shares += (double)job.f.nranks * job.f.m[0] * job.f.m[1] * job.f.m[2] * job.f.n * job.f.n * job.f.n;
    if (job.shares_left == 0) t.finishing.push_back(id);
    else still.push_back(id);
  }
  if (still.size() != s->running.size()) {
    s->running.swap(still);
    s->set_changed = true;
  }
  s->nticks++;
  s->in_flight++;
  return FACES_OK;
}

int submit_at(faces_server *s, const faces_job *j, double t_submit, long long *id)
{
  size_t bytes = 0;
  if (int rc = validate(s, j, &bytes)) return rc;
  Job job;
  job.id = s->next_id++;
  job.spec = *j;
  job.bytes = bytes;
  job.t_submit = t_submit;
  s->jobs.emplace(job.id, job);
  s->queue.push_back(job.id);
  s->submitted++;
  if (id) *id = job.id;
  return FACES_OK;
}

// retire, admit, launch; with wait, block on the oldest tick when no launch
// is possible
int poll(faces_server *s, bool wait, int *ndone)
{
  if (int rc = retire(s, false, ndone)) return rc;
  if (int rc = admit_queued(s)) return rc;
  if (s->running.empty() && s->in_flight == 0 && !s->queue.empty())
    return fail(FACES_ENOMEM,
                "server: queued job %lld (%zu bytes) cannot be admitted: %zu of the %zu-byte budget is held by "
                "done jobs that were not released",
                s->queue.front(), s->jobs[s->queue.front()].bytes, s->resident, s->budget);
  if (!s->running.empty() && s->in_flight < kDepth) return launch_tick(s);
  if (wait && s->in_flight > 0) {
    if (int rc = retire(s, true, ndone)) return rc;
    if (int rc = admit_queued(s)) return rc;
    if (!s->running.empty() && s->in_flight < kDepth) return launch_tick(s);
  }
  return FACES_OK;
}

bool idle(const faces_server *s) { return s->queue.empty() && s->running.empty() && s->in_flight == 0; }

int find_job(faces_server *s, long long id, Job **out)
{
  if (!s) return fail(FACES_EINVAL, "null server");
  auto it = s->jobs.find(id);
  if (it == s->jobs.end()) return fail(FACES_EINVAL, "unknown job %lld", id);
  *out = &it->second;
  return FACES_OK;
}

}  // namespace

extern "C" {

int faces_server_create(faces_server **out, size_t budget_bytes, int max_jobs, unsigned flags)
{
  if (!out) return fail(FACES_EINVAL, "null output pointer");
  if (budget_bytes == 0) return fail(FACES_EINVAL, "budget must be positive");
  if (flags & ~(FACES_SERVE_PLAIN | FACES_SERVE_RELEASE_DONE)) return fail(FACES_EINVAL, "flags 0x%x", flags);
  faces_server *s = new (std::nothrow) faces_server();
  if (!s) return fail(FACES_ENOMEM, "host allocation failed");
  s->budget = budget_bytes;
  s->max_jobs = max_jobs;
  s->flags = flags;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = batch_configure();
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->fetch_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) {
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    e = cudaMemPoolCreate(&s->pool, &props);
  }
  if (e == cudaSuccess) {
    // keep freed memory in the pool: admissions reuse it without the driver
    unsigned long long keep = ~0ull;
    e = cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  for (int i = 0; i < kDepth && e == cudaSuccess; i++) e = cudaEventCreate(&s->ticks[i].ev);
  if (e == cudaSuccess) e = cudaEventCreate(&s->base);
  if (e == cudaSuccess) e = cudaEventRecord(s->base, s->stream);
  if (e == cudaSuccess) e = cudaEventSynchronize(s->base);
  if (e != cudaSuccess) {
    faces_server_destroy(s);
    return fail(FACES_ECUDA, "faces_server_create: %s", cudaGetErrorString(e));
  }
  s->base_host = host_seconds();
  *out = s;
  return FACES_OK;
}

int faces_server_submit(faces_server *s, const faces_job *job, long long *job_id)
{
  if (!s) return fail(FACES_EINVAL, "null server");
  return submit_at(s, job, host_seconds(), job_id);
}

int faces_server_poll(faces_server *s, int wait)
{
  if (!s) return fail(FACES_EINVAL, "null server");
  int ndone = 0;
  if (int rc = poll(s, wait != 0, &ndone)) return rc;
  return ndone;
}

int faces_server_drain(faces_server *s)
{
  if (!s) return fail(FACES_EINVAL, "null server");
  int ndone = 0;
  while (!idle(s))
    if (int rc = poll(s, true, &ndone)) return rc;
  return ndone;
}

int faces_server_job_status(faces_server *s, long long id, int *state, int *shares_done, double *wait_s,
                            double *latency_s)
{
  Job *j = nullptr;
  if (int rc = find_job(s, id, &j)) return rc;
  if (state) *state = j->state;
  if (shares_done) *shares_done = j->shares_done;
  if (wait_s) *wait_s = j->state >= kRunning ? j->t_admit - j->t_submit : -1.0;
  if (latency_s) *latency_s = j->state >= kDone ? j->t_done - j->t_submit : -1.0;
  return FACES_OK;
}

int faces_server_field(faces_server *s, long long id, double **u, long *total_doubles)
{
  Job *j = nullptr;
  if (int rc = find_job(s, id, &j)) return rc;
  if (j->state == kQueued || j->state == kReleased)
    return fail(FACES_EINVAL, "job %lld has no field (queued or released)", id);
  if (u) *u = j->f.u;
  if (total_doubles) *total_doubles = (long)(j->bytes / sizeof(double));
  return FACES_OK;
}

int faces_server_fetch(faces_server *s, long long id, double *host_out)
{
  Job *j = nullptr;
  if (int rc = find_job(s, id, &j)) return rc;
  if (j->state != kDone) return fail(FACES_EINVAL, "job %lld is not done (state %d)", id, j->state);
  if (!host_out) return fail(FACES_EINVAL, "null host buffer");
  // a done job's field is final: no later tick touches it
  CUDA_TRY(cudaMemcpyAsync(host_out, j->f.u, j->bytes, cudaMemcpyDeviceToHost, s->fetch_stream), "server: fetch");
  CUDA_TRY(cudaStreamSynchronize(s->fetch_stream), "server: fetch");
  return FACES_OK;
}

int faces_server_release(faces_server *s, long long id)
{
  Job *j = nullptr;
  if (int rc = find_job(s, id, &j)) return rc;
  if (j->state != kDone && j->state != kReleased)
    return fail(FACES_EINVAL, "job %lld is not done (state %d)", id, j->state);
  if (int rc = release_job(s, *j)) return rc;
  s->jobs.erase(id);
  return FACES_OK;
}

int faces_server_tune(faces_server *s, int unit_div, int run, int half)
{
  if (!s) return fail(FACES_EINVAL, "null server");
  if (half > 2) return fail(FACES_EINVAL, "half = %d: 0, 1 or 2", half);
  if (half >= 0) s->half = half;
  if (unit_div > 0) s->unit_div = unit_div;
  if (run > 0) s->run = run;
  s->set_changed = true;
  return FACES_OK;
}

int faces_server_tune_warp(faces_server *s, int max_n, int boost)
{
  if (!s) return fail(FACES_EINVAL, "null server");
  if (max_n > kBatchWarpMaxN) return fail(FACES_EINVAL, "max_n = %d: at most %d", max_n, kBatchWarpMaxN);
  if (max_n >= 0) s->warp_n = max_n;
  if (boost > 0) s->boost = boost;
  s->set_changed = true;
  return FACES_OK;
}

int faces_server_stats(const faces_server *s, faces_serve_stats *st)
{
  if (!s || !st) return fail(FACES_EINVAL, "null argument");
  st->submitted = s->submitted;
  st->admitted = s->admitted;
  st->completed = s->completed;
  st->ticks = s->nticks;
  st->launches = s->launches;
  st->job_shares = s->job_shares;
  st->point_shares = s->point_shares;
  st->resident_bytes = s->resident;
  st->peak_resident_bytes = s->peak_resident;
  st->budget_bytes = s->budget;
  st->queued = (int)s->queue.size();
  st->running = (int)s->running.size();
  return FACES_OK;
}

int faces_server_run_trace(faces_server *s, int njobs, const faces_job *jobs, const double *arrival_s,
                           long long *job_ids, double *latency_s, double *makespan_s)
{
  if (!s || njobs < 0 || (njobs > 0 && (!jobs || !arrival_s))) return fail(FACES_EINVAL, "bad trace arguments");
  for (int i = 1; i < njobs; i++)
    if (arrival_s[i] < arrival_s[i - 1]) return fail(FACES_EINVAL, "arrival times must not decrease");
  std::vector<long long> ids(njobs, 0);
  const double t0 = host_seconds();
  int next = 0;
  while (next < njobs || !idle(s)) {
    const double now = host_seconds() - t0;
    // arrivals up to now, each stamped with its scheduled arrival time
    while (next < njobs && arrival_s[next] <= now) {
      if (int rc = submit_at(s, &jobs[next], t0 + arrival_s[next], &ids[next])) return rc;
      next++;
    }
    if (idle(s)) {
      // nothing to run: sleep until shortly before the next arrival
      const double dt = arrival_s[next] - (host_seconds() - t0);
      if (dt > 2e-4) std::this_thread::sleep_for(std::chrono::duration<double>(dt - 1e-4));
      continue;
    }
    // block on the oldest tick only when the pipeline is full or nothing
    // else can start
    const bool full = s->in_flight >= kDepth || (s->running.empty() && s->queue.empty());
    if (int rc = poll(s, full, nullptr)) return rc;
  }
  if (makespan_s) *makespan_s = host_seconds() - t0;
  for (int i = 0; i < njobs; i++) {
    if (job_ids) job_ids[i] = ids[i];
    if (latency_s) {
      auto it = s->jobs.find(ids[i]);
      latency_s[i] = it != s->jobs.end() ? it->second.t_done - it->second.t_submit : -1.0;
    }
  }
  return FACES_OK;
}

int faces_server_destroy(faces_server *s)
{
  if (!s) return FACES_OK;
  if (s->stream) {
    cudaStreamSynchronize(s->stream);
    for (auto &kv : s->jobs)
      if (kv.second.f.u) cudaFreeAsync(kv.second.f.u, s->stream);
    for (auto &kv : s->nbr_cache) cudaFreeAsync(kv.second.first, s->stream);
    if (s->d_tables) cudaFreeAsync(s->d_tables, s->stream);
    cudaStreamSynchronize(s->stream);
  }
  for (auto &t : s->ticks) {
    if (t.ev) cudaEventDestroy(t.ev);
    if (t.staging) cudaFreeHost(t.staging);
  }
  if (s->base) cudaEventDestroy(s->base);
  if (s->pool) cudaMemPoolDestroy(s->pool);
  if (s->stream) cudaStreamDestroy(s->stream);
  if (s->fetch_stream) cudaStreamDestroy(s->fetch_stream);
  delete s;
  return FACES_OK;
}

}  // extern "C"
