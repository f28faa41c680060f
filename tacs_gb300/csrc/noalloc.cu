// Compliance / KS-failure evaluation that performs no device allocation.
//
// Intended for callers that own all device memory themselves and may not
// call cudaMalloc: e.g. a host framework that hands this library views into
// its own pre-allocated arena, or a time-stepping / optimisation loop that
// has frozen its memory footprint and where an allocation (which can
// implicitly synchronise the device) is not allowed.  The caller passes
// every input and the output; the only working memory is the file-scope
// array below, sized for at most TG_NOALLOC_MAX_ELEMENTS elements.
#include <cmath>
#include <mutex>
#include <string>

#include "tg_internal.h"

namespace {

// Per element: nq failure values, nq detXd weights and one strain energy
// (nq = 8 for hex8, 4 for MITC4), then the reduction partials and scalars.
constexpr int kMaxNq = 8;
constexpr int kPartials = 256;
constexpr size_t kScratchDoubles =
    (size_t)TG_NOALLOC_MAX_ELEMENTS * (2 * kMaxNq + 1) + kPartials + 8;

// Shared by every call on a device and kept between calls; calls that
// overlap on the GPU (e.g. on two streams) race on it.
static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
static double *g_scratch_ptr[kMaxDevices] = {nullptr};
static std::mutex g_setup_lock;

// Device address of the scratch array for the current device.  The host
// symbol is only a stand-in: the address must come from
// cudaGetSymbolAddress, once per device, with that device current.
int scratch_for_current_device(double **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return tg::cuda_check(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) {
    tg::set_error("tg_eval_functions_noalloc: device ordinal out of range");
    return TG_ERR_ARG;
  }
  std::lock_guard<std::mutex> guard(g_setup_lock);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return tg::cuda_check(e, "cudaGetSymbolAddress");
    g_scratch_ptr[dev] = static_cast<double *>(p);
  }
  *out = g_scratch_ptr[dev];
  return 0;
}

__global__ void finalize_funcs_kernel(const double *scalars, double ksw,
                                      double *vals) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    vals[0] = scalars[0];
    vals[1] = scalars[1] + log(scalars[2]) / ksw;
  }
}

}  // namespace

extern "C" int tg_eval_functions_noalloc(
    int elem_type, int num_elements, const int *conn, const double *xpts,
    const double *thick, double E, double nu, double ys, int transform,
    const double *ref_axis_host, const double *vars, double ks_weight,
    double *vals, void *stream) {
  using namespace tg;
  if (elem_type != TG_ELEM_MITC4 && elem_type != TG_ELEM_HEX8) {
    set_error("tg_eval_functions_noalloc: unknown element type");
    return TG_ERR_ARG;
  }
  if (num_elements < 1 || num_elements > TG_NOALLOC_MAX_ELEMENTS) {
    set_error("tg_eval_functions_noalloc: num_elements must be in [1, "
              "TG_NOALLOC_MAX_ELEMENTS = " +
              std::to_string(TG_NOALLOC_MAX_ELEMENTS) + "]");
    return TG_ERR_ARG;
  }
  if (!conn || !xpts || !thick || !vars || !vals || !(ks_weight > 0.0) ||
      (transform == 1 && !ref_axis_host)) {
    set_error("tg_eval_functions_noalloc: NULL input/output or bad KS weight");
    return TG_ERR_ARG;
  }
  double *scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc) return rc;

  ElemParams ep{};
  ep.elem_type = elem_type;
  ep.rho = 0.0;
  ep.E = E;
  ep.nu = nu;
  ep.ys = ys;
  ep.transform = transform;
  ep.ref_axis[0] = 1.0;
  if (transform == 1) {
    double nrm = std::sqrt(ref_axis_host[0] * ref_axis_host[0] +
                           ref_axis_host[1] * ref_axis_host[1] +
                           ref_axis_host[2] * ref_axis_host[2]);
    double inv = nrm != 0.0 ? 1.0 / nrm : 0.0;
    for (int k = 0; k < 3; k++) ep.ref_axis[k] = ref_axis_host[k] * inv;
  }
  const int nq = elem_type == TG_ELEM_MITC4 ? 4 : 8;
  const size_t ne = (size_t)num_elements;
  double *fail = scratch;
  double *wdet = fail + ne * nq;
  double *sed = wdet + ne * nq;
  double *partials = sed + ne;
  double *scalars = partials + kPartials;

  MeshView m{};
  m.nelem = num_elements;
  m.vpn = elem_type == TG_ELEM_MITC4 ? 6 : 3;
  m.npe = elem_type == TG_ELEM_MITC4 ? 4 : 8;
  m.conn = conn;
  m.xpts = xpts;
  m.thick = thick;
  cudaStream_t s = (cudaStream_t)stream;
  // every scratch entry read below is written first in this call
  if (elem_type == TG_ELEM_MITC4)
    launch_shell_points(ep, m, vars, fail, wdet, sed, s);
  else
    launch_hex_points(ep, m, vars, fail, wdet, sed, s);
  launch_reduce_sum(sed, ne, partials, kPartials, scalars, s);
  launch_reduce_max(fail, ne * nq, partials, kPartials, scalars + 1, s);
  launch_ks_sum(fail, wdet, ne * nq, scalars + 1, ks_weight, partials,
                kPartials, scalars + 2, s);
  finalize_funcs_kernel<<<1, 32, 0, s>>>(scalars, ks_weight, vals);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_check(e, "tg_eval_functions_noalloc");
  return 0;
}
