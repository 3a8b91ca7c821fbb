// The request loop behind ajg_submit / ajg_poll / ajg_wait / ajg_cancel /
// ajg_render_batch, and the FP64 image-error reduction.
//
// One host thread per context owns a stream, a multi-job wave arena and the
// per-wave tables.  It admits queued jobs while the HBM budget allows
// (scenes + arena + films + result buffers), plans each wave from the
// running jobs (one chunk per job and wave: a pixel range of the job's
// current sample pass, or several whole passes of its window when they fit),
// uploads the tables, launches the wave's bounce loop as one CUDA graph
// (cached per bounce count and triangle test) and then the resolves and
// copies of the results that wave completes.  Up to `inflight_waves` waves
// are queued ahead; results are handed over when their wave's event fires.
//
// A pixel's samples always reach its film in sample order: a job's passes
// are scheduled in order, a job appears at most once per wave, and waves run
// in stream order.  So the film -- and the image -- of a job is the same
// bit for bit as rendering it alone with ajg_render.
#include <algorithm>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <thread>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "scene.cuh"

// the layouts the ctypes binding and the header comments state
static_assert(sizeof(ajg_job_desc) == 224, "ajg_job_desc layout");
static_assert(sizeof(ajg_job_status) == 56, "ajg_job_status layout");
static_assert(sizeof(ajg_serve_opts) == 16, "ajg_serve_opts layout");
static_assert(sizeof(ajg_serve_stats) == 88, "ajg_serve_stats layout");
static_assert(sizeof(ajg_scene_info) == 56, "ajg_scene_info layout");
static_assert(sizeof(ajg_emitter) == 32, "ajg_emitter layout");
static_assert(sizeof(ajg_sppm_params) == 40, "ajg_sppm_params layout");

namespace ajg {
namespace {

double now_ms(const ajg_ctx* ctx) {
  return std::chrono::duration<double, std::milli>(
             std::chrono::steady_clock::now() - ctx->t0)
      .count();
}

int fail(ajg_ctx* ctx, int code, const std::string& m) {
  ctx->last_error = m;
  return code;
}

struct Job {
  uint64_t id = 0;
  ajg_scene* scene = nullptr;
  ajg_camera cam{};
  ajg_render_params prm{};
  JobParams jp{};
  uint32_t npix = 0;
  uint32_t progress = 0;
  float* out_host = nullptr;
  float* out_user_dev = nullptr;
  // device (request-loop stream)
  float4* film = nullptr;  // float32 sum + compensation, or float64 sum
  float4* out_dev = nullptr;
  bool own_out = false;
  uint64_t bytes = 0;  // admission charge
  // schedule cursor: the pass of samples [s_cur, s_cur + pass_S) has been
  // handed out for pixels [0, pix_cur)
  uint32_t s_cur = 0, pix_cur = 0, pass_S = 0;
  int inflight = 0;  // waves on the GPU that use the film
  bool admitted = false, started = false, cancel = false, ended = false;
  // status (under the server mutex)
  ajg_job_status st{};
};

// One result hand-over: the job's window resolved after a wave.
struct Report {
  Job* job;
  uint32_t spp;
  bool final_;
  size_t staging_off;  // host copy: offset into the staging ring
  size_t bytes;
  char* dedicated;     // or a pinned buffer of its own
};

struct InFlight {
  cudaEvent_t ev0 = nullptr;  // recorded before the wave's work
  cudaEvent_t ev;
  std::vector<Job*> jobs;
  std::vector<Report> reports;
  uint32_t* err;  // pinned word: the wave's device guard
};

// Pinned host staging for result copies, allocated and freed in FIFO order.
struct StagingRing {
  char* base = nullptr;
  size_t cap = 0, head = 0, used = 0;
  std::deque<std::pair<size_t, size_t>> live;  // (offset, bytes incl. pad)
  bool alloc(size_t bytes, size_t* off) {
    if (!base || bytes > cap) return false;
    size_t start = head;
    size_t pad = 0;
    if (start + bytes > cap) {  // wrap: waste the tail
      pad = cap - start;
      start = 0;
    }
    if (used + pad + bytes > cap) return false;
    used += pad + bytes;
    head = start + bytes;
    if (head == cap) head = 0;
    live.emplace_back(start, pad + bytes);
    *off = start;
    return true;
  }
  void free_oldest() {
    if (live.empty()) return;
    used -= live.front().second;
    live.pop_front();
    if (live.empty()) head = used = 0;
  }
};

constexpr size_t kStagingBytes = 512ull << 20;

}  // namespace

struct Server {
  ajg_ctx* ctx;
  std::thread th;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  bool stop = false;
  ajg_serve_opts opts{AJG_SCHED_FAIR, 256, 2, 0};
  uint64_t want_P = 0;  // wave size the next arena gets (0: the context's)
  uint64_t next_id = 1;
  std::deque<Job*> pending;
  std::vector<Job*> active;  // admitted, not ended (admission order)
  std::unordered_map<uint64_t, Job*> jobs;
  ajg_serve_stats stats{};
  int init_rc = AJG_OK;
  std::string init_error;

  // request-loop thread only
  cudaStream_t st = nullptr;
  // the trace stream of the waves' overlapped closest-hit launches
  cudaStream_t ts = nullptr;
  cudaEvent_t ev_queue = nullptr, ev_hits = nullptr;
  void* arena = nullptr;
  uint64_t arena_bytes = 0, P = 0;
  int NT = 0;
  WaveBufs w{};
  char* d_tables = nullptr;
  MJTables t{};
  std::vector<char*> h_tables;  // pinned, one per in-flight slot + 1
  size_t table_bytes = 0;
  uint64_t wave_no = 0;
  std::map<std::tuple<int, int, int, bool>, cudaGraphExec_t> graphs;
  std::deque<InFlight> inflight;
  std::vector<uint32_t*> err_words;  // pinned, recycled
  uint32_t* d_err = nullptr;
  TraceCounters* d_ctr = nullptr;
  StagingRing ring;

  explicit Server(ajg_ctx* c) : ctx(c) {}

  void run();
  bool admit_locked();
  bool plan_and_launch();
  void retire_oldest();
  void end_job_locked(Job* j, uint32_t state, int err);
  int ensure_arena(int nt, uint64_t target_paths);
  cudaGraphExec_t graph_for(int bounces, int tri_test, int width, bool emit);
};

namespace {

size_t align256(size_t b) { return (b + 255) / 256 * 256; }

// The request loop's default wave (its arena counts against the HBM
// admission budget): the context's wave size, at most 32 Mi paths.
uint64_t serve_default_paths(const ajg_ctx* ctx) {
  return std::min<uint64_t>(ctx->wave_paths, 1u << 25);
}

size_t tables_size() {
  return align256(sizeof(WaveHeader)) +
         align256(sizeof(DeviceScene) * kMaxWaveChunks) +
         align256(sizeof(JobRec) * kMaxWaveChunks) +
         align256(sizeof(Chunk) * kMaxWaveChunks);
}

}  // namespace

int Server::ensure_arena(int nt, uint64_t target) {
  if (arena && nt <= NT && P == target) return AJG_OK;
  // a bigger light count needs a bigger arena: drain, then regrow
  while (!inflight.empty()) retire_oldest();
  for (auto& g : graphs) cudaGraphExecDestroy(g.second);
  graphs.clear();
  if (arena) cudaFree(arena);
  arena = nullptr;
  P = target;
  NT = std::max(nt, NT > 0 ? NT : 3);
  arena_bytes = wave_bytes(P, NT, true);
  if (cudaMalloc(&arena, arena_bytes) != cudaSuccess) {
    arena = nullptr;
    arena_bytes = 0;
    return AJG_ERR_OOM;
  }
  w = carve_wave(static_cast<char*>(arena), P, NT, true);
  return AJG_OK;
}

cudaGraphExec_t Server::graph_for(int bounces, int tri_test, int width,
                                  bool emit) {
  const auto key = std::make_tuple(bounces, tri_test, width, emit);
  auto it = graphs.find(key);
  if (it != graphs.end()) return it->second;
  prepare_mj_kernels();
  cudaGraph_t g = nullptr;
  cudaGraphExec_t ex = nullptr;
  if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) !=
      cudaSuccess)
    return nullptr;
  enqueue_mj_wave(t, w, P, NT, bounces, tri_test, width, emit, d_ctr, d_err,
                  st, ctx->overlap ? ts : nullptr, ev_queue, ev_hits,
                  ctx->packet_camera, ctx->packet_shadow > 0);
  if (cudaStreamEndCapture(st, &g) != cudaSuccess || !g) return nullptr;
  if (cudaGraphInstantiate(&ex, g, 0) != cudaSuccess) ex = nullptr;
  cudaGraphDestroy(g);
  if (ex) {
    graphs[key] = ex;
    ++stats.graph_builds;
  }
  return ex;
}

// Under mu.  Frees the job's device buffers (stream-ordered after every wave
// that used them) and publishes its final state.
void Server::end_job_locked(Job* j, uint32_t state, int err) {
  if (j->ended) return;
  j->ended = true;
  if (j->film) cudaFreeAsync(j->film, st);
  if (j->own_out && j->out_dev) cudaFreeAsync(j->out_dev, st);
  j->film = nullptr;
  j->out_dev = nullptr;
  if (j->admitted) stats.active_bytes -= j->bytes;
  j->st.state = state;
  j->st.error = err;
  j->st.done_ms = now_ms(ctx);
  if (state == AJG_JOB_DONE) ++stats.jobs_done;
  if (state == AJG_JOB_CANCELLED) ++stats.jobs_cancelled;
  if (state == AJG_JOB_FAILED) ++stats.jobs_failed;
  active.erase(std::remove(active.begin(), active.end(), j), active.end());
  j->scene->jobs.fetch_sub(1);
  cv_done.notify_all();
}

// Under mu.  Admits queued jobs in arrival order while slots and the HBM
// budget allow.
bool Server::admit_locked() {
  bool any = false;
  const uint32_t max_active =
      std::min<uint32_t>(opts.max_active_jobs ? opts.max_active_jobs : 256,
                         kMaxWaveChunks);
  while (!pending.empty() && active.size() < max_active) {
    Job* j = pending.front();
    if (j->cancel) {
      pending.pop_front();
      end_job_locked(j, AJG_JOB_CANCELLED, AJG_ERR_CANCELLED);
      continue;
    }
    const uint64_t budget = ctx->hbm_budget;
    // the wave arena counts from the first admission on, allocated or not
    const uint64_t arena_need = std::max<uint64_t>(
        arena_bytes,
        wave_bytes(want_P ? want_P : serve_default_paths(ctx),
                   std::max(3, (int)j->jp.nl + 1), true));
    const uint64_t held =
        ctx->resident_bytes + arena_need + stats.active_bytes;
    if (budget && held + j->bytes > budget) {
      if (active.empty()) {  // can never fit
        pending.pop_front();
        j->st.error = AJG_ERR_OOM;
        end_job_locked(j, AJG_JOB_FAILED, AJG_ERR_OOM);
        continue;
      }
      break;  // wait for running jobs to free their films
    }
    const uint64_t film_bytes = (uint64_t)j->npix * 32;
    void* film = nullptr;
    if (cudaMallocAsync(&film, film_bytes, st) != cudaSuccess) {
      pending.pop_front();
      end_job_locked(j, AJG_JOB_FAILED, AJG_ERR_OOM);
      continue;
    }
    cudaMemsetAsync(film, 0, film_bytes, st);
    j->film = static_cast<float4*>(film);
    if (j->out_user_dev) {
      j->out_dev = reinterpret_cast<float4*>(j->out_user_dev);
    } else {
      void* o = nullptr;
      if (cudaMallocAsync(&o, (uint64_t)j->npix * 16, st) != cudaSuccess) {
        cudaFreeAsync(film, st);
        j->film = nullptr;
        pending.pop_front();
        end_job_locked(j, AJG_JOB_FAILED, AJG_ERR_OOM);
        continue;
      }
      j->out_dev = static_cast<float4*>(o);
      j->own_out = true;
    }
    pending.pop_front();
    j->admitted = true;
    stats.active_bytes += j->bytes;
    active.push_back(j);
    any = true;
  }
  return any;
}

namespace {

struct Plan {
  Job* job;
  uint32_t pix0, n_pix, S, s0;
  bool report, final_;
};

// One chunk of `j` within `budget` paths of a `P`-path wave, advancing its
// cursor.  A pass runs to the next multiple of the progress interval (or to
// the last sample), at most P samples per pixel; without progressive
// results a chunk may cover several passes of the whole window.
bool take(Job* j, uint64_t budget, uint64_t P, Plan* out) {
  const uint32_t spp = j->prm.spp;
  if (j->s_cur >= spp || budget == 0) return false;
  const uint32_t pe = j->progress ? j->progress : spp;
  const uint32_t rem = spp - j->s_cur;
  const uint32_t s0 = j->s_cur, pix0 = j->pix_cur;
  uint32_t S, n;
  if (j->pix_cur == 0) {
    const uint32_t next_b = std::min(spp, (j->s_cur / pe + 1) * pe);
    j->pass_S = (uint32_t)std::min<uint64_t>(next_b - j->s_cur, P);
    const uint64_t whole = budget / j->npix;  // samples for every pixel
    if (whole >= j->pass_S) {
      // several passes at once only when no result is due in between
      S = j->progress ? j->pass_S : (uint32_t)std::min<uint64_t>(rem, whole);
      n = j->npix;
      j->s_cur += S;
    } else {
      S = j->pass_S;
      n = (uint32_t)std::min<uint64_t>(j->npix, budget / S);
      if (n == 0) return false;
      j->pix_cur = n;
      if (j->pix_cur == j->npix) {
        j->pix_cur = 0;
        j->s_cur += S;
      }
    }
  } else {
    S = j->pass_S;
    n = (uint32_t)std::min<uint64_t>(j->npix - j->pix_cur, budget / S);
    if (n == 0) return false;
    j->pix_cur += n;
    if (j->pix_cur == j->npix) {
      j->pix_cur = 0;
      j->s_cur += S;
    }
  }
  const bool pass_done = j->pix_cur == 0;
  const bool fin = pass_done && j->s_cur == spp;
  const bool report =
      pass_done && (fin || (j->progress && s0 / pe != j->s_cur / pe));
  *out = Plan{j, pix0, n, S, s0, report, fin};
  return true;
}

uint64_t remaining_paths(const Job* j) {
  const uint64_t done = (uint64_t)j->s_cur * j->npix +
                        (uint64_t)j->pix_cur * j->pass_S;
  return (uint64_t)j->prm.spp * j->npix - done;
}

}  // namespace

// Plans one wave from the running jobs and enqueues it.  False when there
// is no work to launch.
bool Server::plan_and_launch() {
  std::vector<Plan> plan;
  int bounces = 0, tri_test = -1, width = 0, nt_max = 1;
  uint64_t target_P = 0;
  {
    std::lock_guard<std::mutex> lk(mu);
    target_P = want_P ? want_P : serve_default_paths(ctx);
    for (Job* j : active) {
      if (j->cancel || j->s_cur >= j->prm.spp) continue;
      if (tri_test < 0) {
        tri_test = (int)j->scene->d.tri_test;
        width = (int)j->scene->d.width;
      }
      nt_max = std::max(nt_max, (int)j->jp.nl + 1);
    }
    if (tri_test < 0) return false;
  }
  if (ensure_arena(nt_max, target_P) != AJG_OK) {
    std::lock_guard<std::mutex> lk(mu);
    std::vector<Job*> fail_jobs;
    for (Job* j : active)
      if (j->inflight == 0) fail_jobs.push_back(j);
    for (Job* j : fail_jobs) end_job_locked(j, AJG_JOB_FAILED, AJG_ERR_OOM);
    return false;
  }
  {
    std::lock_guard<std::mutex> lk(mu);
    std::vector<Job*> cand;
    for (Job* j : active) {
      if (j->cancel || j->s_cur >= j->prm.spp) continue;
      // one triangle test and node width per wave (the oldest job's);
      // arena light terms
      if ((int)j->scene->d.tri_test != tri_test ||
          (int)j->scene->d.width != width)
        continue;
      if ((int)j->jp.nl + 1 > NT) continue;
      cand.push_back(j);
    }
    if (cand.empty()) return false;
    uint64_t cap = P;
    std::vector<char> got(cand.size(), 0);
    if (opts.policy == AJG_SCHED_FAIR) {
      // processor sharing: water-fill the wave over the jobs' remaining work
      std::vector<std::pair<uint64_t, size_t>> want;
      for (size_t i = 0; i < cand.size(); ++i)
        want.emplace_back(remaining_paths(cand[i]), i);
      std::sort(want.begin(), want.end());
      std::vector<uint64_t> alloc(cand.size(), 0);
      uint64_t left = cap;
      size_t n_left = want.size();
      for (auto& wj : want) {
        const uint64_t a = std::min(wj.first, left / n_left);
        alloc[wj.second] = a;
        left -= a;
        --n_left;
      }
      for (size_t i = 0; i < cand.size(); ++i) {  // admission order
        Plan p;
        if (take(cand[i], std::min(alloc[i], cap), P, &p)) {
          plan.push_back(p);
          got[i] = 1;
          cap -= (uint64_t)p.n_pix * p.S;
        }
      }
    }
    // FIFO, or what the fair shares left over
    for (size_t i = 0; i < cand.size() && cap; ++i) {
      Plan p;
      if (got[i]) continue;
      if (take(cand[i], cap, P, &p)) {
        plan.push_back(p);
        got[i] = 1;
        cap -= (uint64_t)p.n_pix * p.S;
      }
    }
    if (plan.empty()) return false;
    const double t = now_ms(ctx);
    for (auto& p : plan) {
      bounces = std::max(bounces, (int)p.job->jp.max_b);
      ++p.job->inflight;
      if (!p.job->started) {
        p.job->started = true;
        p.job->st.state = AJG_JOB_RUNNING;
        p.job->st.start_ms = t;
      }
    }
  }

  // tables: scenes of the wave, one record per job, one chunk per job
  char* h = h_tables[wave_no % h_tables.size()];
  WaveHeader* hdr = reinterpret_cast<WaveHeader*>(h);
  char* cur = h + align256(sizeof(WaveHeader));
  DeviceScene* hs = reinterpret_cast<DeviceScene*>(cur);
  cur += align256(sizeof(DeviceScene) * kMaxWaveChunks);
  JobRec* hj = reinterpret_cast<JobRec*>(cur);
  cur += align256(sizeof(JobRec) * kMaxWaveChunks);
  Chunk* hc = reinterpret_cast<Chunk*>(cur);
  std::unordered_map<const ajg_scene*, uint32_t> scene_idx;
  uint32_t n_sc = 0, path_off = 0, pix_off = 0;
  for (size_t i = 0; i < plan.size(); ++i) {
    const Plan& p = plan[i];
    Job* j = p.job;
    auto it = scene_idx.find(j->scene);
    uint32_t si;
    if (it == scene_idx.end()) {
      si = n_sc++;
      scene_idx[j->scene] = si;
      hs[si] = j->scene->d;
    } else {
      si = it->second;
    }
    JobRec& r = hj[i];
    std::memset(&r, 0, sizeof(r));
    r.j = j->jp;
    r.cam = j->cam;
    r.scene = si;
    if (j->prm.flags & AJG_RENDER_FP64_FILM) {
      r.fsum64 = reinterpret_cast<double*>(j->film);
    } else {
      r.fsum = j->film;
      r.fcomp = j->film + j->npix;
    }
    hc[i] = Chunk{(uint32_t)i, p.pix0, p.n_pix, p.S, p.s0, path_off, pix_off, 0};
    path_off += p.n_pix * p.S;
    pix_off += p.n_pix;
  }
  hdr->n_chunks = (uint32_t)plan.size();
  hdr->n_paths = path_off;
  hdr->n_pix = pix_off;
  hdr->n_jobs = (uint32_t)plan.size();
  hdr->n_scenes = n_sc;
  hdr->cap_paths = (uint32_t)P;
  cudaMemcpyAsync(d_tables, h, table_bytes, cudaMemcpyHostToDevice, st);

  InFlight f{};
  cudaEventCreate(&f.ev0);
  cudaEventRecord(f.ev0, st);
  // the closest-hit MIS BSDF pass runs when a scene of the wave has emitters
  bool emit = false;
  for (const Plan& p : plan) emit |= p.job->scene->d.tri_emit != nullptr;
  cudaGraphExec_t g = graph_for(bounces, tri_test, width, emit);
  if (g) {
    cudaGraphLaunch(g, st);
  } else {  // capture unavailable: the same launches on the stream
    cudaGetLastError();
    enqueue_mj_wave(t, w, P, NT, bounces, tri_test, width, emit, d_ctr, d_err,
                    st, ctx->overlap ? ts : nullptr, ev_queue, ev_hits,
                    ctx->packet_camera, ctx->packet_shadow > 0);
  }
  // results this wave completes
  for (const Plan& p : plan) {
    f.jobs.push_back(p.job);
    if (!p.report) continue;
    Job* j = p.job;
    enqueue_resolve(j->film, j->film + j->npix,
                    (j->prm.flags & AJG_RENDER_FP64_FILM)
                        ? reinterpret_cast<const double*>(j->film)
                        : nullptr,
                    j->jp.win_w, j->jp.win_h, j->jp.x0 == 0, j->jp.y0 == 0,
                    j->out_dev, st);
    Report r{j, p.s0 + p.S, p.final_, 0, 0, nullptr};
    if (j->out_host) {
      r.bytes = (size_t)j->npix * 16;
      if (!ring.base && cudaHostAlloc((void**)&ring.base, kStagingBytes,
                                      cudaHostAllocDefault) == cudaSuccess)
        ring.cap = kStagingBytes;
      while (!ring.alloc(r.bytes, &r.staging_off)) {
        if (r.bytes > ring.cap || inflight.empty()) {
          cudaHostAlloc((void**)&r.dedicated, r.bytes, cudaHostAllocDefault);
          break;
        }
        retire_oldest();
      }
      char* dst = r.dedicated ? r.dedicated : ring.base + r.staging_off;
      cudaMemcpyAsync(dst, j->out_dev, r.bytes, cudaMemcpyDeviceToHost, st);
    }
    f.reports.push_back(r);
  }
  if (err_words.empty()) {
    uint32_t* e = nullptr;
    cudaHostAlloc((void**)&e, sizeof(uint32_t), cudaHostAllocDefault);
    err_words.push_back(e);
  }
  f.err = err_words.back();
  err_words.pop_back();
  *f.err = 0;
  cudaMemcpyAsync(f.err, d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
  cudaMemsetAsync(d_err, 0, sizeof(uint32_t), st);
  cudaEventCreate(&f.ev);
  cudaEventRecord(f.ev, st);
  {
    std::lock_guard<std::mutex> lk(mu);
    ++stats.waves;
    stats.paths += path_off;
    stats.kernel_launches +=
        mj_wave_kernels(bounces, emit, width, ctx->packet_shadow > 0) +
        f.reports.size();
  }
  inflight.push_back(std::move(f));
  ++wave_no;
  return true;
}

// Waits for the oldest wave, hands over its results and retires jobs.
void Server::retire_oldest() {
  if (inflight.empty()) return;
  InFlight f = std::move(inflight.front());
  inflight.pop_front();
  cudaEventSynchronize(f.ev);
  float wave_ms = 0.f;
  if (f.ev0 && cudaEventElapsedTime(&wave_ms, f.ev0, f.ev) != cudaSuccess) {
    cudaGetLastError();
    wave_ms = 0.f;
  }
  if (f.ev0) cudaEventDestroy(f.ev0);
  cudaEventDestroy(f.ev);
  const uint32_t guard = *f.err;
  err_words.push_back(f.err);
  std::lock_guard<std::mutex> lk(mu);
  stats.busy_ms += wave_ms;
  // host copies out of the staging memory, under the lock so that
  // ajg_job_read sees whole results
  for (const Report& r : f.reports) {
    if (r.job->out_host && (r.dedicated || ring.base)) {
      const char* src = r.dedicated ? r.dedicated : ring.base + r.staging_off;
      if (!r.job->cancel && !r.job->ended && !guard)
        std::memcpy(r.job->out_host, src, r.bytes);
      if (r.dedicated)
        cudaFreeHost(r.dedicated);
      else
        ring.free_oldest();
    }
  }
  const double t = now_ms(ctx);
  for (const Report& r : f.reports) {
    Job* j = r.job;
    if (j->ended || j->cancel || guard) continue;
    j->st.spp_done = r.spp;
    ++j->st.updates;
    ++stats.results_delivered;
    if (j->st.updates == 1) j->st.first_result_ms = t;
  }
  for (Job* j : f.jobs) {
    --j->inflight;
    if (j->ended) continue;
    if (guard) {
      end_job_locked(j, AJG_JOB_FAILED, AJG_ERR_DEVICE);
      continue;
    }
    if (j->inflight == 0 && j->cancel) {
      end_job_locked(j, AJG_JOB_CANCELLED, AJG_ERR_CANCELLED);
      continue;
    }
    if (j->inflight == 0 && j->st.spp_done == j->prm.spp)
      end_job_locked(j, AJG_JOB_DONE, AJG_OK);
  }
  cv_done.notify_all();
}

void Server::run() {
  cudaSetDevice(ctx->device);
  for (;;) {
    bool have_work = false;
    {
      std::unique_lock<std::mutex> lk(mu);
      admit_locked();
      // cancelled jobs with nothing on the GPU end here
      for (size_t i = 0; i < active.size();) {
        Job* j = active[i];
        if (j->cancel && j->inflight == 0) {
          end_job_locked(j, AJG_JOB_CANCELLED, AJG_ERR_CANCELLED);
          continue;
        }
        ++i;
      }
      if (stop && inflight.empty()) break;
      for (Job* j : active)
        if (!j->cancel && j->s_cur < j->prm.spp) have_work = true;
      if (!have_work && inflight.empty()) {
        cv_work.wait(lk, [&] { return stop || !pending.empty(); });
        continue;
      }
    }
    const uint32_t max_inflight = std::max<uint32_t>(1, opts.inflight_waves);
    if (inflight.size() >= max_inflight) retire_oldest();
    bool launched = false;
    if (have_work && !stop) launched = plan_and_launch();
    if (!launched && !inflight.empty()) retire_oldest();
    // hand over what already finished without blocking
    while (!inflight.empty() &&
           cudaEventQuery(inflight.front().ev) == cudaSuccess)
      retire_oldest();
  }
  // shutdown: end every job still known
  std::lock_guard<std::mutex> lk(mu);
  while (!pending.empty()) {
    Job* j = pending.front();
    pending.pop_front();
    end_job_locked(j, AJG_JOB_CANCELLED, AJG_ERR_CANCELLED);
  }
  while (!active.empty())
    end_job_locked(active.front(), AJG_JOB_CANCELLED, AJG_ERR_CANCELLED);
}

// Starts the request loop on first use.
static int ensure_server(ajg_ctx* ctx, Server** out) {
  std::lock_guard<std::mutex> lk(ctx->server_mu);
  if (!ctx->server) {
    cudaSetDevice(ctx->device);
    auto* s = new Server(ctx);
    bool ok = cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking) ==
                  cudaSuccess &&
              cudaStreamCreateWithFlags(&s->ts, cudaStreamNonBlocking) ==
                  cudaSuccess &&
              cudaEventCreateWithFlags(&s->ev_queue, cudaEventDisableTiming) ==
                  cudaSuccess &&
              cudaEventCreateWithFlags(&s->ev_hits, cudaEventDisableTiming) ==
                  cudaSuccess &&
              cudaMalloc(&s->d_err, sizeof(uint32_t)) == cudaSuccess &&
              cudaMalloc(&s->d_ctr, 2 * sizeof(TraceCounters)) == cudaSuccess;
    s->table_bytes = tables_size();
    ok = ok && cudaMalloc(&s->d_tables, s->table_bytes) == cudaSuccess;
    if (ok) {
      cudaMemset(s->d_err, 0, sizeof(uint32_t));
      cudaMemset(s->d_ctr, 0, 2 * sizeof(TraceCounters));
      cudaMemset(s->d_tables, 0, s->table_bytes);
      char* cur = s->d_tables;
      s->t.hdr = reinterpret_cast<const WaveHeader*>(cur);
      cur += align256(sizeof(WaveHeader));
      s->t.scenes = reinterpret_cast<const DeviceScene*>(cur);
      cur += align256(sizeof(DeviceScene) * kMaxWaveChunks);
      s->t.jobs = reinterpret_cast<const JobRec*>(cur);
      cur += align256(sizeof(JobRec) * kMaxWaveChunks);
      s->t.chunks = reinterpret_cast<const Chunk*>(cur);
      s->t.err = s->d_err;
      // in-flight slots: the default depth plus one; deeper settings reuse
      // them only after their wave retired (retire_oldest runs first)
      for (int i = 0; i < 9 && ok; ++i) {
        char* h = nullptr;
        ok = cudaHostAlloc((void**)&h, s->table_bytes, cudaHostAllocDefault) ==
             cudaSuccess;
        if (ok) s->h_tables.push_back(h);
      }
    }
    if (!ok) {
      cudaGetLastError();
      for (char* h : s->h_tables) cudaFreeHost(h);
      if (s->d_tables) cudaFree(s->d_tables);
      if (s->d_err) cudaFree(s->d_err);
      if (s->d_ctr) cudaFree(s->d_ctr);
      if (s->st) cudaStreamDestroy(s->st);
      if (s->ts) cudaStreamDestroy(s->ts);
      if (s->ev_queue) cudaEventDestroy(s->ev_queue);
      if (s->ev_hits) cudaEventDestroy(s->ev_hits);
      delete s;
      return fail(ctx, AJG_ERR_OOM, "request loop: allocation failed");
    }
    s->th = std::thread([s] { s->run(); });
    ctx->server = s;
  }
  *out = ctx->server;
  return AJG_OK;
}

// Waits for the request loop's queued GPU work (before freeing a scene).
void server_sync(ajg_ctx* ctx) {
  std::lock_guard<std::mutex> lk(ctx->server_mu);
  if (ctx->server) cudaStreamSynchronize(ctx->server->st);
}

void server_shutdown(ajg_ctx* ctx) {
  Server* s = nullptr;
  {
    std::lock_guard<std::mutex> lk(ctx->server_mu);
    s = ctx->server;
    ctx->server = nullptr;
  }
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    for (Job* j : s->active) j->cancel = true;
    for (Job* j : s->pending) j->cancel = true;
  }
  s->cv_work.notify_all();
  s->th.join();
  cudaStreamSynchronize(s->st);
  for (auto& g : s->graphs) cudaGraphExecDestroy(g.second);
  for (char* h : s->h_tables) cudaFreeHost(h);
  for (uint32_t* e : s->err_words) cudaFreeHost(e);
  if (s->ring.base) cudaFreeHost(s->ring.base);
  if (s->arena) cudaFree(s->arena);
  cudaFree(s->d_tables);
  cudaFree(s->d_err);
  cudaFree(s->d_ctr);
  cudaStreamSynchronize(s->ts);
  cudaEventDestroy(s->ev_queue);
  cudaEventDestroy(s->ev_hits);
  cudaStreamDestroy(s->ts);
  cudaStreamDestroy(s->st);
  for (auto& kv : s->jobs) delete kv.second;
  delete s;
}

namespace {

__global__ void k_rmse_partial(const float4* __restrict__ a, uint32_t sa,
                               const float4* __restrict__ b, uint32_t sb,
                               uint32_t w, uint32_t h, double* part_sum,
                               unsigned long long* part_n) {
  __shared__ double ssum[256];
  __shared__ unsigned long long sn[256];
  double acc = 0.0;
  unsigned long long n = 0;
  const uint64_t total = (uint64_t)w * h;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t x = (uint32_t)(i % w), y = (uint32_t)(i / w);
    const float4 pa = a[(uint64_t)y * sa + x], pb = b[(uint64_t)y * sb + x];
    if (!(pa.w > 0.f) || !(pb.w > 0.f)) continue;
    if (!(isfinite(pa.x) && isfinite(pa.y) && isfinite(pa.z) &&
          isfinite(pb.x) && isfinite(pb.y) && isfinite(pb.z)))
      continue;  // pixels holding a NaN or inf sample
    const double ia = 1.0 / pa.w, ib = 1.0 / pb.w;
    const double dx = pa.x * ia - pb.x * ib;
    const double dy = pa.y * ia - pb.y * ib;
    const double dz = pa.z * ia - pb.z * ib;
    acc += dx * dx + dy * dy + dz * dz;
    ++n;
  }
  ssum[threadIdx.x] = acc;
  sn[threadIdx.x] = n;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) {
      ssum[threadIdx.x] += ssum[threadIdx.x + o];
      sn[threadIdx.x] += sn[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part_sum[blockIdx.x] = ssum[0];
    part_n[blockIdx.x] = sn[0];
  }
}

Job* find_job(Server* s, uint64_t id) {
  auto it = s->jobs.find(id);
  return it == s->jobs.end() ? nullptr : it->second;
}

}  // namespace
}  // namespace ajg

using namespace ajg;

extern "C" {

int ajg_serve_configure(ajg_ctx* ctx, const ajg_serve_opts* opts) {
  if (!ctx || !opts) return AJG_ERR_INVALID;
  if (opts->policy > AJG_SCHED_FIFO)
    return ajg::fail(ctx, AJG_ERR_INVALID, "unknown scheduling policy");
  if (opts->max_active_jobs > (uint32_t)kMaxWaveChunks)
    return ajg::fail(ctx, AJG_ERR_INVALID, "max_active_jobs above 1024");
  if (opts->inflight_waves > 8)
    return ajg::fail(ctx, AJG_ERR_INVALID, "inflight_waves above 8");
  if (opts->wave_paths && (opts->wave_paths < 1024 || opts->wave_paths > (1u << 27)))
    return ajg::fail(ctx, AJG_ERR_INVALID, "wave_paths must be in [1024, 2^27]");
  Server* s = nullptr;
  int rc = ensure_server(ctx, &s);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(s->mu);
  s->opts = *opts;
  if (!s->opts.inflight_waves) s->opts.inflight_waves = 2;
  s->want_P = opts->wave_paths;
  return AJG_OK;
}

int ajg_submit(ajg_ctx* ctx, const ajg_job_desc* d, uint64_t* job_id) {
  if (!ctx) return AJG_ERR_INVALID;
  if (!d || !job_id || !d->scene)
    return ajg::fail(ctx, AJG_ERR_INVALID, "NULL argument");
  if (d->scene->ctx != ctx)
    return ajg::fail(ctx, AJG_ERR_INVALID, "scene of another context");
  int rc = check_render(ctx, d->scene->d, d->camera, d->params);
  if (rc) return rc;
  uint32_t x0 = d->window[0], y0 = d->window[1], ww = d->window[2],
           wh = d->window[3];
  if (ww == 0 || wh == 0) {
    x0 = y0 = 0;
    ww = d->camera.width;
    wh = d->camera.height;
  }
  if ((uint64_t)x0 + ww > d->camera.width ||
      (uint64_t)y0 + wh > d->camera.height)
    return ajg::fail(ctx, AJG_ERR_INVALID, "window outside the film");
  const uint64_t npix = (uint64_t)ww * wh;
  Server* s = nullptr;
  rc = ensure_server(ctx, &s);
  if (rc) return rc;
  auto* j = new Job();
  j->scene = d->scene;
  j->cam = d->camera;
  j->prm = d->params;
  j->jp = make_job_params(d->scene, d->camera, d->params);
  j->jp.x0 = x0;
  j->jp.y0 = y0;
  j->jp.win_w = ww;
  j->jp.win_h = wh;
  j->npix = (uint32_t)npix;
  j->progress = d->progress_spp;
  j->out_host = d->out_rgbw;
  j->out_user_dev = d->d_out_rgbw;
  j->bytes = npix * 32 + (d->d_out_rgbw ? 0 : npix * 16);
  j->st.state = AJG_JOB_QUEUED;
  j->st.spp_total = d->params.spp;
  j->st.submit_ms = now_ms(ctx);
  d->scene->jobs.fetch_add(1);
  {
    std::lock_guard<std::mutex> lk(s->mu);
    j->id = s->next_id++;
    s->jobs[j->id] = j;
    s->pending.push_back(j);
    ++s->stats.jobs_submitted;
  }
  s->cv_work.notify_all();
  *job_id = j->id;
  return AJG_OK;
}

int ajg_poll(ajg_ctx* ctx, uint64_t id, ajg_job_status* out) {
  if (!ctx || !out) return AJG_ERR_INVALID;
  Server* s = ctx->server;
  if (!s) return ajg::fail(ctx, AJG_ERR_NOT_FOUND, "unknown job");
  std::lock_guard<std::mutex> lk(s->mu);
  Job* j = find_job(s, id);
  if (!j) return ajg::fail(ctx, AJG_ERR_NOT_FOUND, "unknown job");
  *out = j->st;
  return AJG_OK;
}

int ajg_wait(ajg_ctx* ctx, uint64_t id, int32_t timeout_ms,
             ajg_job_status* out) {
  if (!ctx) return AJG_ERR_INVALID;
  Server* s = ctx->server;
  if (!s) return ajg::fail(ctx, AJG_ERR_NOT_FOUND, "unknown job");
  std::unique_lock<std::mutex> lk(s->mu);
  Job* j = find_job(s, id);
  if (!j) return ajg::fail(ctx, AJG_ERR_NOT_FOUND, "unknown job");
  auto ended = [&] { return j->ended; };
  if (timeout_ms < 0)
    s->cv_done.wait(lk, ended);
  else
    s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ended);
  if (out) *out = j->st;
  if (!j->ended) return AJG_ERR_TIMEOUT;
  if (j->st.state == AJG_JOB_DONE) return AJG_OK;
  if (j->st.state == AJG_JOB_CANCELLED) return AJG_ERR_CANCELLED;
  return j->st.error ? j->st.error : AJG_ERR_DEVICE;
}

int ajg_job_read(ajg_ctx* ctx, uint64_t id, float* out_rgbw,
                 ajg_job_status* out) {
  if (!ctx) return AJG_ERR_INVALID;
  Server* s = ctx->server;
  if (!s) return ajg::fail(ctx, AJG_ERR_NOT_FOUND, "unknown job");
  std::lock_guard<std::mutex> lk(s->mu);
  Job* j = find_job(s, id);
  if (!j) return ajg::fail(ctx, AJG_ERR_NOT_FOUND, "unknown job");
  if (out_rgbw) {
    if (!j->out_host)
      return ajg::fail(ctx, AJG_ERR_INVALID, "job has no host result buffer");
    std::memcpy(out_rgbw, j->out_host, (size_t)j->npix * 16);
  }
  if (out) *out = j->st;
  return AJG_OK;
}

int ajg_cancel(ajg_ctx* ctx, uint64_t id) {
  if (!ctx) return AJG_ERR_INVALID;
  Server* s = ctx->server;
  if (!s) return ajg::fail(ctx, AJG_ERR_NOT_FOUND, "unknown job");
  {
    std::lock_guard<std::mutex> lk(s->mu);
    Job* j = find_job(s, id);
    if (!j) return ajg::fail(ctx, AJG_ERR_NOT_FOUND, "unknown job");
    if (!j->ended) j->cancel = true;
  }
  s->cv_work.notify_all();
  return AJG_OK;
}

int ajg_job_release(ajg_ctx* ctx, uint64_t id) {
  if (!ctx) return AJG_ERR_INVALID;
  Server* s = ctx->server;
  if (!s) return ajg::fail(ctx, AJG_ERR_NOT_FOUND, "unknown job");
  std::lock_guard<std::mutex> lk(s->mu);
  Job* j = find_job(s, id);
  if (!j) return ajg::fail(ctx, AJG_ERR_NOT_FOUND, "unknown job");
  if (!j->ended)
    return ajg::fail(ctx, AJG_ERR_INVALID, "job has not ended");
  s->jobs.erase(id);
  delete j;
  return AJG_OK;
}

int ajg_render_batch(ajg_ctx* ctx, const ajg_job_desc* jobs, uint32_t n,
                     ajg_job_status* status) {
  if (!ctx || (n && !jobs)) return AJG_ERR_INVALID;
  std::vector<uint64_t> ids;
  int first = AJG_OK;
  for (uint32_t i = 0; i < n; ++i) {
    uint64_t id = 0;
    const int rc = ajg_submit(ctx, &jobs[i], &id);
    if (rc) {
      for (uint64_t k : ids) ajg_cancel(ctx, k);
      for (uint64_t k : ids) {
        ajg_wait(ctx, k, -1, nullptr);
        ajg_job_release(ctx, k);
      }
      return rc;
    }
    ids.push_back(id);
  }
  for (uint32_t i = 0; i < n; ++i) {
    ajg_job_status st{};
    const int rc = ajg_wait(ctx, ids[i], -1, &st);
    if (status) status[i] = st;
    if (rc && !first) first = rc;
    ajg_job_release(ctx, ids[i]);
  }
  return first;
}

int ajg_serve_get_stats(ajg_ctx* ctx, ajg_serve_stats* out) {
  if (!ctx || !out) return AJG_ERR_INVALID;
  Server* s = ctx->server;
  std::memset(out, 0, sizeof(*out));
  if (!s) return AJG_OK;
  std::lock_guard<std::mutex> lk(s->mu);
  *out = s->stats;
  return AJG_OK;
}

int ajg_image_rmse(ajg_ctx* ctx, const float* d_a, uint32_t stride_a,
                   const float* d_b, uint32_t stride_b, uint32_t width,
                   uint32_t height, double* rmse, uint64_t* pixels) {
  if (!ctx) return AJG_ERR_INVALID;
  if (!d_a || !d_b || !rmse)
    return ajg::fail(ctx, AJG_ERR_INVALID, "NULL argument");
  if (stride_a < width || stride_b < width)
    return ajg::fail(ctx, AJG_ERR_INVALID, "stride below width");
  std::lock_guard<std::mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  constexpr int kBlocks = kSMs * 4;
  double* d_sum = nullptr;
  unsigned long long* d_n = nullptr;
  if (cudaMallocAsync((void**)&d_sum, kBlocks * sizeof(double), ctx->stream) !=
          cudaSuccess ||
      cudaMallocAsync((void**)&d_n, kBlocks * sizeof(unsigned long long),
                      ctx->stream) != cudaSuccess)
    return ajg::fail(ctx, AJG_ERR_OOM, "image_rmse: allocation failed");
  k_rmse_partial<<<kBlocks, 256, 0, ctx->stream>>>(
      reinterpret_cast<const float4*>(d_a), stride_a,
      reinterpret_cast<const float4*>(d_b), stride_b, width, height, d_sum,
      d_n);
  ++ctx->kernel_launches;
  std::vector<double> hs(kBlocks);
  std::vector<unsigned long long> hn(kBlocks);
  cudaMemcpyAsync(hs.data(), d_sum, kBlocks * sizeof(double),
                  cudaMemcpyDeviceToHost, ctx->stream);
  cudaMemcpyAsync(hn.data(), d_n, kBlocks * sizeof(unsigned long long),
                  cudaMemcpyDeviceToHost, ctx->stream);
  cudaFreeAsync(d_sum, ctx->stream);
  cudaFreeAsync(d_n, ctx->stream);
  const cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess)
    return ajg::fail(ctx, AJG_ERR_CUDA,
                     std::string("image_rmse: ") + cudaGetErrorString(e));
  double acc = 0.0;
  unsigned long long n = 0;
  for (int i = 0; i < kBlocks; ++i) {  // fixed order: deterministic
    acc += hs[i];
    n += hn[i];
  }
  *rmse = n ? std::sqrt(acc / (3.0 * (double)n)) : 0.0;
  if (pixels) *pixels = n;
  return AJG_OK;
}

}  // extern "C"
