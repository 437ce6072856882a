// Serving loop: XC builds of many molecules through one GPU with continuous
// batching and admission against a device-memory budget.
//
// OCC's compute_vxc is a blocking call on one molecule (include/occ/dft/dft.h
// :395-429); a service in front of it sees a stream of molecules, each going
// through its SCF iterations.  Here a client opens a session per molecule
// (the host part -- grid, leaves, screening -- is built on the caller's
// thread), then submits one density per iteration and collects V_xc / E_xc
// by ticket.  One worker thread owns the GPU: every tick it takes the oldest
// pending build of up to max_batch admitted sessions (at most one per
// session, so a session's builds run in submission order) and runs them as
// one mixed-precision launch sequence (or one FP64 build after the other).
// A session is admitted -- its device state materialised -- only while the
// sum of the admitted sessions' device bytes stays within the budget; a
// session that does not fit waits (later, smaller ones may go first), one
// that could never fit is refused at open.  An admitted session keeps its
// grid, weights, screening lists and its per-build workspace, AO values
// included, resident until it closes: the AO values are computed on its first
// build only.  The workspaces are carved from one device pool that one TMA
// tensor map covers, so builds of any set of sessions share launches.
// Closing a session frees its device state once its builds are done.
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

#include "xc_engine.hpp"

namespace occx {
namespace {

using Clock = std::chrono::steady_clock;

thread_local std::string t_server_error;

struct Session {
  uint64_t id = 0;
  std::unique_ptr<Molecule> mol;
  double charge = 0.0; // admission charge: resident device bytes (upper bound) + ws
  size_t ws = 0;       // workspace at the server's precision (AO values resident)
  size_t ws_off = 0;   // its place in the pool while admitted
  bool ao_valid = false;
  bool admitted = false;
  bool closing = false;
  long queued = 0; // builds submitted and not yet run
};

struct Job {
  uint64_t ticket = 0, session = 0;
  std::vector<double> D, V;
  double exc2[2] = {0.0, 0.0};
  Clock::time_point submitted, finished;
  int status = 1; // 1 pending, OCC_XC_OK done, < 0 failed
  std::string err;
};

// First-fit allocator of 512-byte-aligned ranges of the workspace pool.
struct PoolAlloc {
  std::map<size_t, size_t> free_; // offset -> bytes
  void reset(size_t bytes) {
    free_.clear();
    if (bytes)
      free_[0] = bytes;
  }
  bool alloc(size_t bytes, size_t &off) {
    bytes = (bytes + 511) / 512 * 512;
    for (auto it = free_.begin(); it != free_.end(); ++it)
      if (it->second >= bytes) {
        off = it->first;
        const size_t rest = it->second - bytes;
        free_.erase(it);
        if (rest)
          free_[off + bytes] = rest;
        return true;
      }
    return false;
  }
  void release(size_t off, size_t bytes) {
    bytes = (bytes + 511) / 512 * 512;
    auto it = free_.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
};

double pct(std::vector<double> v, double q) {
  if (v.empty())
    return 0.0;
  std::sort(v.begin(), v.end());
  const double pos = q * (v.size() - 1);
  const size_t i = static_cast<size_t>(pos);
  const double f = pos - i;
  return i + 1 < v.size() ? v[i] * (1 - f) + v[i + 1] * f : v[i];
}

} // namespace

struct Server {
  occ_xc_server_settings cfg{};
  int device = 0;
  std::unique_ptr<Context> ctx;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::map<uint64_t, std::unique_ptr<Session>> sessions;
  std::map<uint64_t, std::unique_ptr<Job>> jobs; // ordered by ticket = submission order
  uint64_t next_id = 1;
  long pending = 0;
  double admitted_bytes = 0.0, peak_bytes = 0.0;
  bool stop = false, paused = false;
  std::vector<double> latency_ms;
  long ticks = 0, tick_builds = 0, completed = 0, failed = 0;
  std::string fatal;
  ListArena arena;
  char *pool = nullptr; // the sessions' workspaces (allocated at the first admission)
  size_t pool_size = 0;
  PoolAlloc pool_free;
  WsMaps pool_map;
  int *d_err = nullptr;
  double *h_stage = nullptr; // pinned staging for D in / V out
  size_t stage_cap = 0;      // doubles
  std::thread worker;

  Server(int dev, const occ_xc_server_settings &s) : cfg(s), device(dev) {
    ctx = std::make_unique<Context>(dev);
    cuda_check(cudaMalloc(&d_err, sizeof(int)), "cudaMalloc");
    cuda_check(cudaMemset(d_err, 0, sizeof(int)), "cudaMemset");
    worker = std::thread([this] { run(); });
  }

  ~Server() {
    {
      std::lock_guard<std::mutex> lk(mu);
      stop = true;
    }
    cv_work.notify_all();
    if (worker.joinable())
      worker.join();
    cudaSetDevice(device);
    sessions.clear(); // frees the molecules' device state
    if (h_stage)
      cudaFreeHost(h_stage);
    if (d_err)
      cudaFree(d_err);
    if (pool)
      cudaFree(pool);
  }

  // The pool, at the first admission: settings.pool_bytes, or the budget,
  // capped at 40 % of the device memory free then.
  void ensure_pool() {
    if (pool)
      return;
    size_t fr = 0, tot = 0;
    cuda_check(cudaMemGetInfo(&fr, &tot), "cudaMemGetInfo");
    double want = cfg.pool_bytes > 0 ? cfg.pool_bytes
                                     : std::min(cfg.hbm_budget_bytes, 0.4 * static_cast<double>(fr));
    const size_t bytes = std::max<size_t>(static_cast<size_t>(want) / 512 * 512, 512);
    cuda_check(cudaMalloc(&pool, bytes), "cudaMalloc");
    pool_size = bytes;
    pool_free.reset(bytes);
    encode_ws_map(pool_map, pool, bytes);
  }

  void stage(size_t doubles) {
    if (doubles <= stage_cap)
      return;
    const size_t n = std::max(doubles, 2 * stage_cap);
    if (h_stage)
      cudaFreeHost(h_stage);
    h_stage = nullptr;
    stage_cap = 0;
    cuda_check(cudaMallocHost(&h_stage, n * sizeof(double)), "cudaMallocHost");
    stage_cap = n;
  }

  // Pick this tick's builds; sessions to admit are charged here and
  // materialised by the caller outside the lock.
  void select(std::vector<Job *> &tick, std::vector<Session *> &admit,
              std::vector<std::unique_ptr<Session>> &retire) {
    for (auto it = sessions.begin(); it != sessions.end();) {
      Session &S = *it->second;
      if (S.closing && S.queued == 0) {
        if (S.admitted) {
          admitted_bytes -= S.charge;
          pool_free.release(S.ws_off, S.ws);
        }
        retire.push_back(std::move(it->second));
        it = sessions.erase(it);
      } else {
        ++it;
      }
    }
    if (paused)
      return;
    std::vector<uint64_t> taken;
    for (auto &kv : jobs) {
      Job &J = *kv.second;
      if (J.status != 1 || static_cast<int>(tick.size()) >= cfg.max_batch)
        continue;
      if (std::find(taken.begin(), taken.end(), J.session) != taken.end())
        continue; // one build per session per tick, in submission order
      taken.push_back(J.session);
      Session &S = *sessions.at(J.session);
      if (!S.admitted && S.ws > pool_size) { // can never be admitted
        J.status = OCC_XC_ERR_NOMEM;
        J.err = "the molecule's workspace is larger than the server's device pool";
        J.finished = Clock::now();
        pending--;
        S.queued--;
        failed++;
        cv_done.notify_all();
        continue;
      }
      if (!S.admitted) {
        if (admitted_bytes + S.charge > cfg.hbm_budget_bytes)
          continue; // waits for memory; a smaller session may go first
        if (!pool_free.alloc(S.ws, S.ws_off))
          continue; // no room in the pool yet
        S.admitted = true;
        S.ao_valid = false;
        admitted_bytes += S.charge;
        peak_bytes = std::max(peak_bytes, admitted_bytes);
        admit.push_back(&S);
      }
      tick.push_back(&J);
    }
  }

  void run() {
    if (cudaSetDevice(device) != cudaSuccess) {
      std::lock_guard<std::mutex> lk(mu);
      fatal = "cudaSetDevice failed on the server thread";
      return;
    }
    for (;;) {
      std::vector<Job *> tick;
      std::vector<Session *> admit;
      std::vector<std::unique_ptr<Session>> retire;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv_work.wait(lk, [&] { return stop || work_ready(); });
        if (stop)
          return;
        if (!pool) {
          try {
            ensure_pool();
          } catch (const std::exception &e) {
            fatal = e.what();
            return;
          }
        }
        select(tick, admit, retire);
      }
      retire.clear(); // device memory freed outside the lock
      if (tick.empty()) {
        std::unique_lock<std::mutex> lk(mu);
        // nothing runnable (all waiting for memory, or paused): sleep until
        // a submission, a close or a resume changes that
        cv_work.wait_for(lk, std::chrono::milliseconds(50));
        continue;
      }
      execute(tick, admit);
    }
  }

  bool work_ready() const {
    for (const auto &kv : sessions)
      if (kv.second->closing && kv.second->queued == 0)
        return true;
    return !paused && pending > 0;
  }

  void finish(std::vector<Job *> &tick, int status, const std::string &err) {
    std::lock_guard<std::mutex> lk(mu);
    const auto now = Clock::now();
    for (Job *J : tick) {
      J->status = status;
      J->err = err;
      J->finished = now;
      pending--;
      sessions.at(J->session)->queued--;
      if (status == OCC_XC_OK) {
        completed++;
        latency_ms.push_back(
            std::chrono::duration<double, std::milli>(J->finished - J->submitted).count());
      } else {
        failed++;
      }
    }
    ticks++;
    tick_builds += static_cast<long>(tick.size());
    cv_done.notify_all();
    cv_work.notify_all();
  }

  void execute(std::vector<Job *> &tick, std::vector<Session *> &admit) {
    // materialise newly admitted sessions; one that does not get its memory
    // (the budget is an accounting limit, the device may hold less) is
    // returned to the waiting state and its build fails with NOMEM
    std::vector<uint64_t> failed_sessions;
    for (Session *S : admit) {
      try {
        S->mol->materialise();
      } catch (const std::exception &e) {
        S->mol->release_device();
        std::lock_guard<std::mutex> lk(mu);
        S->admitted = false;
        admitted_bytes -= S->charge;
        pool_free.release(S->ws_off, S->ws);
        failed_sessions.push_back(S->id);
      }
    }
    if (!failed_sessions.empty()) {
      std::vector<Job *> bad, ok;
      for (Job *J : tick)
        (std::find(failed_sessions.begin(), failed_sessions.end(), J->session) !=
                 failed_sessions.end()
             ? bad
             : ok)
            .push_back(J);
      finish(bad, OCC_XC_ERR_NOMEM, "device allocation failed while admitting the molecule");
      tick.swap(ok);
      if (tick.empty())
        return;
    }
    std::vector<Molecule *> mols;
    std::vector<Session *> sess;
    {
      std::lock_guard<std::mutex> lk(mu);
      for (Job *J : tick) {
        sess.push_back(sessions.at(J->session).get());
        mols.push_back(sess.back()->mol.get());
      }
    }
    cudaStream_t st = ctx->stream;
    try {
      size_t total = 0;
      for (Molecule *M : mols)
        total += 2 * static_cast<size_t>(M->basis.nbf) * M->basis.nbf + 2;
      stage(total);
      size_t off = 0;
      std::vector<size_t> at(mols.size());
      for (size_t i = 0; i < mols.size(); i++) {
        Molecule &M = *mols[i];
        const size_t n2 = static_cast<size_t>(M.basis.nbf) * M.basis.nbf;
        at[i] = off;
        std::memcpy(h_stage + off, tick[i]->D.data(), n2 * sizeof(double));
        cuda_check(cudaMemcpyAsync(M.d_D, h_stage + off, n2 * sizeof(double),
                                   cudaMemcpyHostToDevice, st), "cudaMemcpyAsync H2D");
        off += 2 * n2 + 2;
      }
      if (cfg.precision == OCC_XC_MIXED) {
        std::vector<char *> ws;
        std::vector<int> aov;
        for (Session *S : sess) {
          ws.push_back(pool + S->ws_off);
          aov.push_back(S->ao_valid ? 1 : 0);
        }
        mixed_build_in_pool(*ctx, mols, ws, aov, pool, pool_map, arena, d_err, st);
      } else {
        for (Session *S : sess)
          S->mol->build_fp64(S->mol->d_D, S->mol->d_V, S->mol->d_out2, st,
                             reinterpret_cast<double *>(pool + S->ws_off), S->ao_valid);
      }
      for (Session *S : sess)
        S->ao_valid = true; // the launches above left the AO values in place
      for (size_t i = 0; i < mols.size(); i++) {
        Molecule &M = *mols[i];
        const size_t n2 = static_cast<size_t>(M.basis.nbf) * M.basis.nbf;
        cuda_check(cudaMemcpyAsync(h_stage + at[i] + n2, M.d_V, n2 * sizeof(double),
                                   cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync D2H");
        cuda_check(cudaMemcpyAsync(h_stage + at[i] + 2 * n2, M.d_out2, 2 * sizeof(double),
                                   cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync D2H");
      }
      int flag = 0;
      cuda_check(cudaMemcpyAsync(&flag, d_err, sizeof(int), cudaMemcpyDeviceToHost, st),
                 "cudaMemcpyAsync D2H");
      cuda_check(cudaStreamSynchronize(st), "cudaStreamSynchronize");
      if (flag) {
        cuda_check(cudaMemset(d_err, 0, sizeof(int)), "cudaMemset");
        throw TimeoutError("a bounded wait of the tensor-core pipeline gave up");
      }
      for (size_t i = 0; i < mols.size(); i++) {
        const size_t n2 = static_cast<size_t>(mols[i]->basis.nbf) * mols[i]->basis.nbf;
        tick[i]->V.assign(h_stage + at[i] + n2, h_stage + at[i] + 2 * n2);
        tick[i]->exc2[0] = h_stage[at[i] + 2 * n2];
        tick[i]->exc2[1] = h_stage[at[i] + 2 * n2 + 1];
        tick[i]->D.clear();
        tick[i]->D.shrink_to_fit();
      }
      finish(tick, OCC_XC_OK, "");
    } catch (const TimeoutError &e) {
      finish(tick, OCC_XC_ERR_TIMEOUT, e.what());
    } catch (const CudaError &e) {
      {
        std::lock_guard<std::mutex> lk(mu);
        fatal = e.what();
      }
      finish(tick, OCC_XC_ERR_CUDA, e.what());
    } catch (const std::exception &e) {
      finish(tick, OCC_XC_ERR_INTERNAL, e.what());
    }
  }
};

} // namespace occx

using namespace occx;

struct occ_xc_server {
  std::unique_ptr<Server> impl;
};

namespace {
template <typename F> int server_guard(F &&f) {
  try {
    return f();
  } catch (const MethodError &e) {
    t_server_error = e.what();
    return OCC_XC_ERR_METHOD;
  } catch (const ArgError &e) {
    t_server_error = e.what();
    return OCC_XC_ERR_ARG;
  } catch (const CudaError &e) {
    t_server_error = e.what();
    return OCC_XC_ERR_CUDA;
  } catch (const std::bad_alloc &) {
    t_server_error = "host allocation failed";
    return OCC_XC_ERR_NOMEM;
  } catch (const std::exception &e) {
    t_server_error = e.what();
    return OCC_XC_ERR_INTERNAL;
  }
}
} // namespace

extern "C" {

void occ_xc_default_server_settings(occ_xc_server_settings *s) {
  if (!s)
    return;
  s->hbm_budget_bytes = 150e9;
  s->pool_bytes = 0.0;
  s->queue_capacity = 4096;
  s->max_batch = 64;
  s->precision = OCC_XC_MIXED;
}

const char *occ_xc_server_last_error(void) { return t_server_error.c_str(); }

int occ_xc_server_create(int device, const occ_xc_server_settings *settings,
                         occ_xc_server **out) {
  if (!out)
    return OCC_XC_ERR_ARG;
  *out = nullptr;
  occ_xc_server_settings s;
  occ_xc_default_server_settings(&s);
  if (settings)
    s = *settings;
  if (s.hbm_budget_bytes <= 0 || s.queue_capacity <= 0 || s.max_batch <= 0 ||
      (s.precision != OCC_XC_FP64 && s.precision != OCC_XC_MIXED)) {
    t_server_error = "server settings: budget, queue capacity and batch size must be positive";
    return OCC_XC_ERR_ARG;
  }
  return server_guard([&] {
    auto srv = std::make_unique<occ_xc_server>();
    srv->impl = std::make_unique<Server>(device, s);
    *out = srv.release();
    return OCC_XC_OK;
  });
}

void occ_xc_server_destroy(occ_xc_server *srv) { delete srv; }

int occ_xc_server_open(occ_xc_server *srv, int natoms, const int *Z, const double *xyz,
                       int nshells, const int *shell_l, const int *shell_atom,
                       const int *shell_nprim, const double *exponents,
                       const double *coefficients, int pure, const char *method,
                       const occ_xc_grid_settings *grid, const occ_xc_build_settings *build,
                       uint64_t *session) {
  if (!srv || !session)
    return OCC_XC_ERR_ARG;
  return server_guard([&] {
    Server &S = *srv->impl;
    MoleculeArgs a{natoms, Z, xyz, nshells, shell_l, shell_atom, shell_nprim, exponents,
                   coefficients, pure, method, grid, build};
    auto sess = std::make_unique<Session>();
    sess->mol = molecule_host(S.ctx.get(), a); // host work on the caller's thread
    if (S.cfg.precision == OCC_XC_MIXED)
      require_not_mgga(sess->mol->deriv, "a tensor-core (OCC_XC_MIXED) server");
    sess->ws = S.cfg.precision == OCC_XC_MIXED ? sess->mol->mixed_workspace_bytes()
                                               : sess->mol->fp64_workspace_bytes();
    sess->ws = (sess->ws + 511) / 512 * 512;
    sess->charge = sess->mol->estimate_resident_bytes() + static_cast<double>(sess->ws);
    const double cap = S.cfg.pool_bytes > 0 ? std::min(S.cfg.hbm_budget_bytes, S.cfg.pool_bytes)
                                            : S.cfg.hbm_budget_bytes;
    if (sess->charge > S.cfg.hbm_budget_bytes || static_cast<double>(sess->ws) > cap) {
      t_server_error = "molecule needs " + std::to_string(sess->charge / 1e9) +
                       " GB of device memory, more than the server's budget";
      return static_cast<int>(OCC_XC_ERR_NOMEM);
    }
    std::lock_guard<std::mutex> lk(S.mu);
    sess->id = S.next_id++;
    *session = sess->id;
    S.sessions[sess->id] = std::move(sess);
    return static_cast<int>(OCC_XC_OK);
  });
}

int occ_xc_server_submit(occ_xc_server *srv, uint64_t session, const double *D,
                         uint64_t *ticket) {
  if (!srv || !D || !ticket)
    return OCC_XC_ERR_ARG;
  return server_guard([&] {
    Server &S = *srv->impl;
    auto J = std::make_unique<Job>();
    size_t n2 = 0;
    {
      std::lock_guard<std::mutex> lk(S.mu);
      auto it = S.sessions.find(session);
      if (it == S.sessions.end() || it->second->closing)
        throw ArgError("unknown or closed session");
      if (!S.fatal.empty())
        throw CudaError("server stopped after a CUDA error: " + S.fatal);
      if (S.pending >= S.cfg.queue_capacity) {
        t_server_error = "request queue full";
        return static_cast<int>(OCC_XC_ERR_BUSY);
      }
      const int nbf = it->second->mol->basis.nbf;
      n2 = static_cast<size_t>(nbf) * nbf;
    }
    J->D.assign(D, D + n2); // copied outside the lock
    J->session = session;
    J->submitted = Clock::now();
    {
      std::lock_guard<std::mutex> lk(S.mu);
      auto it = S.sessions.find(session);
      if (it == S.sessions.end() || it->second->closing)
        throw ArgError("unknown or closed session");
      if (S.pending >= S.cfg.queue_capacity) {
        t_server_error = "request queue full";
        return static_cast<int>(OCC_XC_ERR_BUSY);
      }
      J->ticket = S.next_id++;
      *ticket = J->ticket;
      it->second->queued++;
      S.pending++;
      S.jobs[J->ticket] = std::move(J);
    }
    S.cv_work.notify_all();
    return static_cast<int>(OCC_XC_OK);
  });
}

static int collect(Server &S, std::map<uint64_t, std::unique_ptr<Job>>::iterator it, double *V,
                   double *exc2) {
  Job &J = *it->second;
  const int st = J.status;
  if (st == OCC_XC_OK) {
    if (V)
      std::memcpy(V, J.V.data(), J.V.size() * sizeof(double));
    if (exc2) {
      exc2[0] = J.exc2[0];
      exc2[1] = J.exc2[1];
    }
  } else {
    t_server_error = J.err;
  }
  S.jobs.erase(it);
  return st;
}

int occ_xc_server_poll(occ_xc_server *srv, uint64_t ticket, double *V, double *exc2, int *done) {
  if (!srv || !done)
    return OCC_XC_ERR_ARG;
  Server &S = *srv->impl;
  std::lock_guard<std::mutex> lk(S.mu);
  auto it = S.jobs.find(ticket);
  if (it == S.jobs.end()) {
    t_server_error = "unknown ticket (never issued or already collected)";
    return OCC_XC_ERR_ARG;
  }
  if (it->second->status == 1) {
    *done = 0;
    return OCC_XC_OK;
  }
  *done = 1;
  return collect(S, it, V, exc2);
}

int occ_xc_server_wait(occ_xc_server *srv, uint64_t ticket, double timeout_s, double *V,
                       double *exc2) {
  if (!srv)
    return OCC_XC_ERR_ARG;
  Server &S = *srv->impl;
  std::unique_lock<std::mutex> lk(S.mu);
  auto it = S.jobs.find(ticket);
  if (it == S.jobs.end()) {
    t_server_error = "unknown ticket (never issued or already collected)";
    return OCC_XC_ERR_ARG;
  }
  Job *J = it->second.get();
  const auto until =
      Clock::now() + std::chrono::microseconds(static_cast<long long>(std::max(0.0, timeout_s) * 1e6));
  if (!S.cv_done.wait_until(lk, until, [&] { return J->status != 1; })) {
    t_server_error = "build not finished within the timeout";
    return OCC_XC_ERR_TIMEOUT;
  }
  it = S.jobs.find(ticket); // another thread may have collected it meanwhile
  if (it == S.jobs.end()) {
    t_server_error = "ticket collected by another caller";
    return OCC_XC_ERR_ARG;
  }
  return collect(S, it, V, exc2);
}

int occ_xc_server_close(occ_xc_server *srv, uint64_t session) {
  if (!srv)
    return OCC_XC_ERR_ARG;
  Server &S = *srv->impl;
  {
    std::lock_guard<std::mutex> lk(S.mu);
    auto it = S.sessions.find(session);
    if (it == S.sessions.end() || it->second->closing) {
      t_server_error = "unknown or closed session";
      return OCC_XC_ERR_ARG;
    }
    it->second->closing = true;
  }
  S.cv_work.notify_all();
  return OCC_XC_OK;
}

int occ_xc_server_pause(occ_xc_server *srv, int paused) {
  if (!srv)
    return OCC_XC_ERR_ARG;
  Server &S = *srv->impl;
  {
    std::lock_guard<std::mutex> lk(S.mu);
    S.paused = paused != 0;
  }
  S.cv_work.notify_all();
  return OCC_XC_OK;
}

int occ_xc_server_session_info(occ_xc_server *srv, uint64_t session, occ_xc_molecule_info *out,
                               int *admitted) {
  if (!srv || !out)
    return OCC_XC_ERR_ARG;
  Server &S = *srv->impl;
  std::lock_guard<std::mutex> lk(S.mu);
  auto it = S.sessions.find(session);
  if (it == S.sessions.end()) {
    t_server_error = "unknown session";
    return OCC_XC_ERR_ARG;
  }
  const Molecule &M = *it->second->mol;
  out->nbf = M.basis.nbf;
  out->natoms = static_cast<int>(M.Z.size());
  out->nshells = static_cast<int>(M.basis.shells.size());
  out->deriv = M.deriv;
  out->npoints = M.plan.npts;
  out->nleaves = static_cast<long>(M.leaves.size());
  out->flops_per_build = M.flops;
  out->device_bytes = it->second->admitted ? M.device_bytes + it->second->ws : 0.0;
  out->workspace_bytes = static_cast<double>(M.fp64_workspace_bytes());
  out->mixed_workspace_bytes = static_cast<double>(M.mixed_workspace_bytes());
  out->resident_bytes = it->second->charge;
  if (admitted)
    *admitted = it->second->admitted ? 1 : 0;
  return OCC_XC_OK;
}

int occ_xc_server_stats_get(occ_xc_server *srv, occ_xc_server_stats *o) {
  if (!srv || !o)
    return OCC_XC_ERR_ARG;
  Server &S = *srv->impl;
  std::lock_guard<std::mutex> lk(S.mu);
  o->completed = S.completed;
  o->failed = S.failed;
  o->pending = S.pending;
  o->ticks = S.ticks;
  o->mean_batch = S.ticks ? static_cast<double>(S.tick_builds) / S.ticks : 0.0;
  o->p50_ms = pct(S.latency_ms, 0.50);
  o->p99_ms = pct(S.latency_ms, 0.99);
  o->max_ms = S.latency_ms.empty() ? 0.0
                                    : *std::max_element(S.latency_ms.begin(), S.latency_ms.end());
  long adm = 0, wait = 0;
  for (const auto &kv : S.sessions)
    (kv.second->admitted ? adm : wait)++;
  o->sessions_admitted = adm;
  o->sessions_waiting = wait;
  o->admitted_bytes = S.admitted_bytes;
  o->peak_admitted_bytes = S.peak_bytes;
  return OCC_XC_OK;
}

} // extern "C"
