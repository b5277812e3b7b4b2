// sprg_spr_size_from_recovered_noalloc: the SPR size-field stage
// (element errors -> size factor -> element sizes -> vertex average) for
// callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc: a simulation code whose memory
// manager reserves the device heap up front for its own pool (a library
// allocation then fails or fragments that pool), or a host thread in the
// middle of an asynchronous pipeline that cannot afford the device-wide
// synchronisation cudaMalloc/cudaFree may imply.  This entry point takes
// every input and output from the caller and keeps its scratch (per-element
// errors and sizes, block partial sums, the three global scalars) in one
// file-scope __device__ array of a fixed size, which every GPU that loads the
// library holds until the process exits.
//
// Set-up: the first call on a device (with that device current) resolves the
// array's device address with cudaGetSymbolAddress; later calls reuse it.
// The first call on a device should therefore come before any stream capture.
// CUDA loads a library's device code lazily by default, so that first call
// is also the moment the module is loaded and the array's memory committed
// on the device: a caller that reserves the device heap for its own pool
// should make the first call before reserving it (or load modules eagerly,
// CUDA_MODULE_LOADING=EAGER).  Later calls commit no memory.
// Every call shares the array and it keeps the last call's contents; calls
// that overlap on the GPU (two streams, two host threads) race on it.
// A CUDA error already pending from the caller's earlier work is left in
// place and reported as SPRG_ECUDA before anything is launched, so this
// call never claims another call's failure as its own.
#include <mutex>

#include "spr_gb300.h"
#include "sprg_internal.h"

namespace {

constexpr long long kMaxElems = SPRG_NOALLOC_MAX_ELEMS;
constexpr long long kPartials = 2 * ((kMaxElems + 255) / 256);  // two sums per 256-thread block
constexpr long long kScratchDoubles = 2 * kMaxElems + kPartials + 4;

// errors [kMaxElems] | element sizes [kMaxElems] | partials | 3 scalars
static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
double* g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device (set up once).
int scratch_on_current_device(double** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return SPRG_ECUDA;
  if (dev < 0 || dev >= kMaxDevices) return SPRG_EINVAL;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) return SPRG_ECUDA;
    g_scratch_addr[dev] = static_cast<double*>(p);
  }
  *out = g_scratch_addr[dev];
  return SPRG_OK;
}

}  // namespace

extern "C" int sprg_spr_size_from_recovered_noalloc(int dim, int64_t n_verts, int64_t n_elems,
                                                    const double* d_coords, const int32_t* d_elem_verts,
                                                    const int32_t* d_vert_elem_offsets,
                                                    const int32_t* d_vert_elems, const double* d_ip, int ncomp,
                                                    const double* d_rec, double adapt_ratio, double* d_size,
                                                    double* size_factor_out, void* stream) {
  if ((dim != 2 && dim != 3) || n_verts <= 0 || n_elems <= 0) return SPRG_EINVAL;
  if (n_elems > kMaxElems || n_verts > INT32_MAX) return SPRG_EINVAL;  // beyond the fixed scratch
  if (ncomp != 3 && ncomp != 9) return SPRG_EINVAL;
  if (!d_coords || !d_elem_verts || !d_vert_elem_offsets || !d_vert_elems || !d_ip || !d_rec || !d_size)
    return SPRG_EINVAL;
  if (!(adapt_ratio > 0)) return SPRG_EINVAL;
  if (cudaPeekAtLastError() != cudaSuccess) return SPRG_ECUDA;  // the caller's pending error, untouched
  double* base = nullptr;
  int rc = scratch_on_current_device(&base);
  if (rc) return rc;
  double* err = base;
  double* esize = base + kMaxElems;
  double* partials = base + 2 * kMaxElems;
  double* out3 = partials + kPartials;

  sprg::DevMesh m{};
  m.dim = dim;
  m.nn = dim + 1;
  m.ne_el = dim == 3 ? 6 : 3;
  m.V = (int)n_verts;
  m.T = (int)n_elems;
  m.xyz = d_coords;
  m.ev = d_elem_verts;
  m.a_off = d_vert_elem_offsets;
  m.a_el = d_vert_elems;
  m.p_off = d_vert_elem_offsets;
  m.p_el = d_vert_elems;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int nb = sprg::error_blocks(m.T);
  double p = 1, d = dim;
  sprg::launch_error_f64(m, d_ip, ncomp, d_rec, err, partials, nb, (2 * d) / (2 * p + d), s);
  sprg::launch_size_factor(partials, nb, 0, adapt_ratio, 0, dim, out3, s);
  sprg::launch_esize_f64(m, err, out3, 0, 0, 0, esize, s);
  sprg::launch_average(m, esize, d_size, s);
  if (cudaGetLastError() != cudaSuccess) return SPRG_ECUDA;
  if (size_factor_out) {
    if (cudaMemcpyAsync(size_factor_out, out3 + 2, sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess)
      return SPRG_ECUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return SPRG_ECUDA;
  }
  return SPRG_OK;
}
