// candmc_hh_recon_qr_noalloc: TSQR + Householder reconstruction of a narrow
// panel without allocating any memory.
//
// Some callers cannot let a library allocate device memory while they run:
// a serving process that budgets all of the GPU's memory when it starts (an
// allocation in the middle of a request could fail, or push a neighbour past
// its share), or a host framework whose own allocator must own every device
// buffer.  For them this entry point uses a fixed scratch area that lives in
// the library itself, in the file-scope device array below.  Every GPU that
// loads the library holds that array (about 3.7 MB) until the process exits.
//
// Limits: 1 <= b <= 32 and b <= m <= 8192 (larger sizes return
// CANDMC_ERR_ARG before any GPU work).  The caller passes A, W and T as for
// candmc_hh_recon_qr.
//
// All calls share the one array and each call leaves its own data in it.  Two
// calls whose work overlaps on the GPU (different streams, or different host
// threads on one device) race on it; serialize them.
//
// The first call on a device does a one-time set-up with that device
// current: it looks up the device address of the array and raises the leaf
// kernel's shared-memory limit.  Make that first call before any stream
// capture begins.  The set-up is guarded by a mutex, so first calls from
// several host threads are safe (the GPU work itself must still not overlap).
//
// The kernels record a numeric failure (a non-finite U^-1 in the sign-choice
// LU) in a status word inside the shared scratch.  This entry point does not
// read that word back, since that would synchronise the caller's stream; the
// next call clears it.  A caller that needs the check tests W and T for
// non-finite values.
#include <mutex>

#include "kernels.cuh"

namespace candmc {

int hr_direct_prealloc(double* A, int64_t lda, int64_t m, int b, double* T, int64_t ldT, double* W,
                       int64_t ldW, double* Qw, double* Rn, double* Q11, double* Q21,
                       unsigned* cnt, double* Uinv, int* d_status, cudaStream_t s);
void hr_prealloc_sizes(int64_t m, int b, int64_t* P, int64_t* nnodes);
int hr_prealloc_setup();

namespace {

constexpr int64_t kMaxRows = 8192;
constexpr int kMaxB = kDirectB;                  // 32
constexpr int64_t kMaxNodes = 64;                // 32 leaves of <= 256 rows -> 63 tree nodes
constexpr int64_t kQwDoubles = kMaxRows * kMaxB;
constexpr int64_t kNodeDoubles = kMaxNodes * kMaxB * kMaxB;
constexpr int64_t kCountWords = kMaxNodes + 1;   // arrival counters + status word
constexpr int64_t kScratchDoubles =
    kQwDoubles + 3 * kNodeDoubles + (int64_t)kMaxB * kMaxB + (kCountWords + 1) / 2 + 1;

// The scratch area.  In host code this name is only a host-side stand-in for
// the device array, never a device address: the address comes from
// cudaGetSymbolAddress in setup_device().
static __device__ __align__(256) double g_hr_scratch[kScratchDoubles];

struct DeviceScratch {
  bool ready = false;
  double* base = nullptr;
};
static DeviceScratch g_dev[64];
static std::mutex g_dev_mutex;

int setup_device(double** base) {
  int dev = 0;
  CANDMC_CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return set_error(CANDMC_ERR_ARG, "device index out of range");
  std::lock_guard<std::mutex> lock(g_dev_mutex);
  if (!g_dev[dev].ready) {
    void* p = nullptr;
    CANDMC_CK(cudaGetSymbolAddress(&p, g_hr_scratch));
    CANDMC_RET(hr_prealloc_setup());
    g_dev[dev].base = static_cast<double*>(p);
    g_dev[dev].ready = true;
  }
  *base = g_dev[dev].base;
  return CANDMC_OK;
}

}  // namespace
}  // namespace candmc

using namespace candmc;

extern "C" int candmc_hh_recon_qr_noalloc(double* A, int64_t lda, int64_t m, int64_t b, double* W,
                                          double* T, void* stream) {
  if (!A || !W || !T || b < 1 || m < b || lda < m)
    return set_error(CANDMC_ERR_ARG, "hh_recon_qr_noalloc: invalid arguments");
  if (b > kMaxB || m > kMaxRows)
    return set_error(CANDMC_ERR_ARG,
                     "hh_recon_qr_noalloc: limited to b <= 32 and m <= 8192 (fixed scratch)");
  int64_t P, nnodes;
  hr_prealloc_sizes(m, (int)b, &P, &nnodes);
  if (nnodes > kMaxNodes) return set_error(CANDMC_ERR_ARG, "hh_recon_qr_noalloc: tree too large");
  double* base = nullptr;
  CANDMC_RET(setup_device(&base));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  double* Qw = base;
  double* Rn = Qw + kQwDoubles;
  double* Q11 = Rn + kNodeDoubles;
  double* Q21 = Q11 + kNodeDoubles;
  double* Uinv = Q21 + kNodeDoubles;
  unsigned* cnt = reinterpret_cast<unsigned*>(Uinv + (int64_t)kMaxB * kMaxB);
  int* status = reinterpret_cast<int*>(cnt + kMaxNodes);
  // the arrival counters and the status word must start at zero on every call
  CANDMC_CK(cudaMemsetAsync(cnt, 0, sizeof(unsigned) * kCountWords, s));
  return hr_direct_prealloc(A, lda, m, (int)b, T, b, W, b, Qw, Rn, Q11, Q21, cnt, Uinv, status, s);
}
