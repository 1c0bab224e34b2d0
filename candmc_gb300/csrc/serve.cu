// Least-squares request server: continuous batching of single-RHS solves on
// one GPU (the request loop around candmc_ls_solve).
//
// Workers are host threads, each owning one CUDA stream.  Requests wait in a
// queue ordered by arrival time; the worker that takes the queue's head admits
// it once (1) its arrival time has come and (2) its device-memory estimate fits
// beside the requests already admitted within the budget.  Admission is
// strictly in arrival order (no overtaking), so a large request is never
// starved by a stream of small ones.  An admitted request runs on its worker's
// stream: copy A and b in from host memory, candmc_ls_solve (factor + Q^T b +
// refinement, with A, Y\R, T and R resident throughout), copy x out.  The
// kernels a request launches depend only on its own sizes and data, so its
// result is bitwise the same alone and among any mix of other requests.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "kernels.cuh"

namespace candmc {

using Clock = std::chrono::steady_clock;

struct Request {
  int64_t id;
  const double* A;
  int64_t lda, m, n;
  const double* bvec;
  double* x;
  double arrival, admit = 0, done_t = 0;
  int64_t bytes;
  int status = -1;     // -1: not finished
  int worker = -1;
  double stats[4] = {0, 0, 0, 0};
};

class Server {
 public:
  Server(double budget, int nworkers, int precision, int64_t b, int max_refine, double tol, int dev)
      : budget_(budget), precision_(precision), b_(b), max_refine_(max_refine), tol_(tol), dev_(dev),
        t0_(Clock::now()) {
    for (int w = 0; w < nworkers; ++w) workers_.emplace_back([this, w] { run(w); });
    nworkers_ = nworkers;
  }

  ~Server() {
    {
      std::lock_guard<std::mutex> g(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto& t : workers_) t.join();
    std::lock_guard<std::mutex> g(mu_);
    for (auto* r : pending_) r->status = CANDMC_ERR_CANCELLED;
    pending_.clear();
    done_cv_.notify_all();
    for (auto& kv : reqs_) delete kv.second;
  }

  double now() const { return std::chrono::duration<double>(Clock::now() - t0_).count(); }

  int submit(const double* A, int64_t lda, int64_t m, int64_t n, const double* bvec, double* x,
             double arrival, int64_t* ticket) {
    auto* r = new Request();
    r->A = A; r->lda = lda; r->m = m; r->n = n; r->bvec = bvec; r->x = x;
    r->arrival = arrival;
    r->bytes = candmc_ls_request_bytes(m, n, b_, precision_);
    std::lock_guard<std::mutex> g(mu_);
    r->id = next_id_++;
    reqs_[r->id] = r;
    *ticket = r->id;
    if ((double)r->bytes > budget_) {
      r->status = set_error(CANDMC_ERR_ALLOC, "request exceeds the server's memory budget");
      r->admit = r->done_t = now();
      done_cv_.notify_all();
      return r->status;
    }
    // keep the queue sorted by (arrival, id); submissions usually come in order
    auto it = pending_.end();
    while (it != pending_.begin() && (*(it - 1))->arrival > arrival) --it;
    pending_.insert(it, r);
    cv_.notify_all();
    return CANDMC_OK;
  }

  int wait(int64_t id, double timeout_s, double* info) {
    std::unique_lock<std::mutex> lk(mu_);
    auto it = reqs_.find(id);
    if (it == reqs_.end()) return set_error(CANDMC_ERR_ARG, "unknown ticket");
    Request* r = it->second;
    auto pred = [&] { return r->status >= 0; };
    if (timeout_s < 0) {
      done_cv_.wait(lk, pred);
    } else if (!done_cv_.wait_for(lk, std::chrono::duration<double>(timeout_s), pred)) {
      return CANDMC_ERR_TIMEOUT;
    }
    if (info) {
      info[0] = r->status;
      info[1] = r->arrival;
      info[2] = r->admit;
      info[3] = r->done_t;
      info[4] = r->stats[0];
      info[5] = r->stats[1];
      info[6] = (double)r->bytes;
      info[7] = r->worker;
    }
    return r->status;
  }

  void stats(double* out) {
    std::lock_guard<std::mutex> g(mu_);
    out[0] = (double)in_use_;
    out[1] = (double)peak_use_;
    out[2] = (double)completed_;
    out[3] = inflight_;
    out[4] = peak_inflight_;
    out[5] = (double)pending_.size();
    out[6] = budget_;
    out[7] = nworkers_;
  }

 private:
  void run(int w) {
    cudaSetDevice(dev_);
    cudaStream_t s = nullptr;
    const bool have_stream = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) == cudaSuccess;
    std::unique_lock<std::mutex> lk(mu_);
    for (;;) {
      if (stop_) break;
      if (pending_.empty()) {
        cv_.wait(lk);
        continue;
      }
      Request* r = pending_.front();
      const double t = now();
      if (r->arrival > t) {
        cv_.wait_for(lk, std::chrono::duration<double>(r->arrival - t));
        continue;
      }
      if ((double)(in_use_ + r->bytes) > budget_) {
        cv_.wait(lk);   // a completion frees memory and notifies
        continue;
      }
      pending_.pop_front();
      in_use_ += r->bytes;
      peak_use_ = std::max(peak_use_, in_use_);
      ++inflight_;
      peak_inflight_ = std::max(peak_inflight_, inflight_);
      r->admit = t;
      r->worker = w;
      lk.unlock();
      cv_.notify_all();   // the next head may fit as well
      const int st = have_stream ? solve(r, s) : set_error(CANDMC_ERR_CUDA, "worker stream");
      lk.lock();
      r->status = st;
      r->done_t = now();
      in_use_ -= r->bytes;
      --inflight_;
      ++completed_;
      done_cv_.notify_all();
      cv_.notify_all();
    }
    lk.unlock();
    if (have_stream) cudaStreamDestroy(s);
  }

  int solve(Request* r, cudaStream_t s) {
    const int64_t m = r->m, n = r->n;
    int rc;
    {
      DevBuf dA, dB, dX;
      CANDMC_RET(dA.alloc(sizeof(double) * m * n, s));
      CANDMC_RET(dB.alloc(sizeof(double) * m, s));
      CANDMC_RET(dX.alloc(sizeof(double) * n, s));
      CANDMC_CK(cudaMemcpy2DAsync(dA.p, sizeof(double) * m, r->A, sizeof(double) * r->lda,
                                  sizeof(double) * m, n, cudaMemcpyHostToDevice, s));
      CANDMC_CK(cudaMemcpyAsync(dB.p, r->bvec, sizeof(double) * m, cudaMemcpyHostToDevice, s));
      rc = candmc_ls_solve(dA.d(), m, m, n, dB.d(), m, 1, dX.d(), n, b_, precision_, max_refine_, tol_,
                           r->stats, s);
      if (rc == CANDMC_OK)
        CANDMC_CK(cudaMemcpyAsync(r->x, dX.p, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    }
    CANDMC_CK(cudaStreamSynchronize(s));
    return rc;
  }

  const double budget_;
  const int precision_;
  const int64_t b_;
  const int max_refine_;
  const double tol_;
  const int dev_;
  const Clock::time_point t0_;
  int nworkers_ = 0;
  std::mutex mu_;
  std::condition_variable cv_, done_cv_;
  std::deque<Request*> pending_;
  std::unordered_map<int64_t, Request*> reqs_;
  std::vector<std::thread> workers_;
  int64_t next_id_ = 0;
  int64_t in_use_ = 0, peak_use_ = 0, completed_ = 0;
  int inflight_ = 0, peak_inflight_ = 0;
  bool stop_ = false;
};

}  // namespace candmc

using namespace candmc;

extern "C" int64_t candmc_ls_request_bytes(int64_t m, int64_t n, int64_t b, int precision) {
  if (m < 1 || n < 1 || b < 1) return 0;
  const int64_t npan = (n + b - 1) / b, nblk = (n + 127) / 128;
  // inputs and resident state: A, Y\R, b, Q^T b, residual, x, T per panel, R^-1 diagonal blocks
  int64_t by = 8 * (2 * m * n + 4 * m + 4 * n + npan * b * b + nblk * 128 * 128);
  // panel: the TSQR leaf/tree workspace of a 32-column sub-panel (leaf Q
  // blocks, per-leaf T, tree-node R and fan-in-4 Q blocks) at the smallest
  // leaf height, and the recursion's b x b temporaries
  by += 8 * (300 * m + 8 * b * b);
  // refinement products: split-K partials of A x (row tiles) and A^T r
  by += 8 * (m + 4 * 152 * 128 + 4 * 152 * n);
  if (precision != CANDMC_PREC_FP64 && g_panel_oz_min_rows > 0 && m >= g_panel_oz_min_rows) {
    // the panels' emulated-FP64 half-panel updates and Gram products: seven
    // BF16 planes of both operands (128 + 96 padded rows) per row of the
    // panel, and the split-K partials (at most two waves of CTAs)
    by += 2 * 7 * (128 + 96) * m + 8 * 128 * b * 2 * 152;
  }
  if (n > b) {
    // trailing update: BF16 slices / FP32 copies / split-K partials of the
    // contraction over the trailing columns
    const int64_t per = precision == CANDMC_PREC_OZAKI ? 16 : (precision == CANDMC_PREC_FP32 ? 8 : 0);
    by += per * m * n + 8 * 128 * n * 64;
  }
  return by + (32ll << 20);
}

extern "C" int candmc_mem_high_water(int reset, uint64_t* bytes) {
  int dev = 0;
  CANDMC_CK(cudaGetDevice(&dev));
  cudaMemPool_t pool;
  CANDMC_CK(cudaDeviceGetDefaultMemPool(&pool, dev));
  if (reset) {
    uint64_t zero = 0;
    CANDMC_CK(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrUsedMemHigh, &zero));
  }
  if (bytes) CANDMC_CK(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemHigh, bytes));
  return CANDMC_OK;
}

extern "C" int candmc_server_create(double budget_bytes, int nworkers, int precision, int64_t b,
                                    int max_refine, double tol, void** out) {
  if (!out || nworkers < 1 || nworkers > 256 || !(budget_bytes > 0) || b < 1 || b > 128 ||
      max_refine < 0 || precision < CANDMC_PREC_FP64 || precision > CANDMC_PREC_FP32)
    return set_error(CANDMC_ERR_ARG, "server_create args");
  int dev = 0;
  CANDMC_CK(cudaGetDevice(&dev));
  try {
    *out = new Server(budget_bytes, nworkers, precision, b, max_refine, tol, dev);
  } catch (...) {
    *out = nullptr;
    return set_error(CANDMC_ERR_ALLOC, "server_create");
  }
  return CANDMC_OK;
}

extern "C" int candmc_server_submit(void* server, const double* A, int64_t lda, int64_t m, int64_t n,
                                    const double* bvec, double* x, double arrival_s, int64_t* ticket) {
  if (!server || !A || !bvec || !x || !ticket || n < 1 || m < n || lda < m)
    return set_error(CANDMC_ERR_ARG, "server_submit args");
  return static_cast<Server*>(server)->submit(A, lda, m, n, bvec, x, arrival_s, ticket);
}

extern "C" int candmc_server_wait(void* server, int64_t ticket, double timeout_s, double* info) {
  if (!server) return set_error(CANDMC_ERR_ARG, "server_wait args");
  return static_cast<Server*>(server)->wait(ticket, timeout_s, info);
}

extern "C" double candmc_server_now(void* server) {
  return server ? static_cast<Server*>(server)->now() : 0.0;
}

extern "C" int candmc_server_stats(void* server, double* out) {
  if (!server || !out) return set_error(CANDMC_ERR_ARG, "server_stats args");
  static_cast<Server*>(server)->stats(out);
  return CANDMC_OK;
}

extern "C" int candmc_server_destroy(void* server) {
  delete static_cast<Server*>(server);
  return CANDMC_OK;
}
