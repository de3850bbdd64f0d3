// rd_noalloc.cu -- field at points for callers that cannot allocate.
//
// rd_field_at_noalloc evaluates the same field kernel as rd_field_at
// (k_field_points, Calc_Field_at_Batch semantics) but allocates nothing: the
// points and the result are device buffers owned by the caller, and every
// piece of working memory of the call -- the one-entry work plan, the
// struct-of-arrays copies of the points and fields, the partial sums of the
// j-chunks and their tickets -- lives in g_noalloc_scratch below, a
// fixed-size array that every GPU loading the library holds until the
// process exits.
//
// Who needs this: host codes whose device memory belongs to another runtime
// (the reference's OpenACC build keeps its particle and staging arrays in
// OpenACC-managed device memory, so a drop-in passes acc_deviceptr of its own
// point buffers), processes that reserve a fixed device-memory budget up front
// and may not grow it afterwards, and latency-critical loops such as the
// Metropolis-Hastings rounds, which evaluate the field about a thousand times
// per time step (the reference found that creating device copies per call
// dominated small batches, src/mod_verlet.F90:43-50).  Such callers create the
// engine once, at set-up, and then call this entry point as often as needed.
//
// Limits and sharing:
//  - at most RD_NOALLOC_MAX_POINTS points per call (larger M is rejected);
//  - set-up happens when an engine is created (rd_noalloc_prepare, called by
//    rd_engine_create with the engine's device current): it loads this file's
//    module -- the array and its kernels -- and the field and planner kernels
//    the call launches, and resolves the device address of the array
//    (cudaGetSymbolAddress).  Under lazy module loading (the CUDA default) that
//    load is where the array's device memory is committed, so it happens
//    before the caller's time-critical loop, never inside a call;
//  - the call runs on the engine's own stream, which is not ordered after the
//    caller's streams: the caller's writes of the points must be complete
//    (device- or stream-synchronised) before the call; the result is complete
//    when the call returns;
//  - all calls share the array and it keeps the last call's contents; the
//    call clears the tickets it needs at zero itself.  Calls that overlap on
//    the GPU (other streams, other engines, other host threads) race on the
//    array: issue them one after another.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/rumdeed_gpu.h"
#include "rd_pair.cuh"

#define RD_NOALLOC_MAX_POINTS 65536
#define RD_NOALLOC_SCRATCH_BYTES (16u << 20)
#define RD_NOALLOC_MAX_DEVICES 64

// Layout of the scratch (offsets in bytes, each 256-aligned).
#define NA_OFF_PLAN 0                                   // PlanEntry[1]
#define NA_OFF_HDR 256                                  // PlanHeader[1]
#define NA_OFF_INTS 512                                 // int npts[1], int zero_off[1]
#define NA_OFF_PTS 1024                                 // 3 x MAX doubles (x, y, z)
#define NA_OFF_FLD (NA_OFF_PTS + 3 * 8 * RD_NOALLOC_MAX_POINTS)   // 3 x MAX doubles
#define NA_OFF_PART (NA_OFF_FLD + 3 * 8 * RD_NOALLOC_MAX_POINTS)  // partials
#define NA_MAX_ITEMS 4096   // the planner lengthens the j-chunks of a call that would need more
#define NA_OFF_TICK (NA_OFF_PART + NA_MAX_ITEMS * 3 * RD_ITILE * 8)
#define NA_END (NA_OFF_TICK + NA_MAX_ITEMS * 4)
static_assert(NA_END <= RD_NOALLOC_SCRATCH_BYTES, "no-alloc scratch layout exceeds the array");

static __device__ __align__(256) unsigned char g_noalloc_scratch[RD_NOALLOC_SCRATCH_BYTES];

// kernels from the other translation units
cudaError_t rd_launch_plan(cudaStream_t st, const DiodeParams* P, const DiodeDyn* Dy, int nslots,
                           int mode, int chunk_rule, int max_items, const int* npts,
                           PlanEntry* plan, PlanHeader* ph);
cudaError_t rd_launch_field_points(int prec, int geom, int grid, cudaStream_t st,
                                   const DiodeParams* P, const Pool& pool, const PlanEntry* plan,
                                   const PlanHeader* ph, const PointSet& pts, double* partial,
                                   int* tickets, double kscale);
cudaError_t rd_preload_field_points(int prec);
cudaError_t rd_preload_plan();
// engine internals needed here (rd_engine.cu)
int rd_engine_view(rd_engine* e, int diode, const DiodeParams** P, const DiodeDyn** Dy, Pool* pool,
                   int* geometry, int* precision, int* grid, double* kscale, cudaStream_t* st,
                   int* device);
int rd_engine_repack(rd_engine* e);
int rd_engine_chunk_rule(rd_engine* e);
int rd_set_error(int code, const char* msg);

namespace {

__global__ void k_na_begin(int* ints, int M, int* tickets, int nt, const double* pos3m, double* x,
                           double* y, double* z) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t == 0) { ints[0] = M; ints[1] = 0; }
  for (int k = t; k < nt; k += gridDim.x * blockDim.x) tickets[k] = 0;
  for (int i = t; i < M; i += gridDim.x * blockDim.x) {
    x[i] = pos3m[3 * i]; y[i] = pos3m[3 * i + 1]; z[i] = pos3m[3 * i + 2];
  }
}

__global__ void k_na_end(int M, const double* fx, const double* fy, const double* fz, double* out3m) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M; i += gridDim.x * blockDim.x) {
    out3m[3 * i] = fx[i]; out3m[3 * i + 1] = fy[i]; out3m[3 * i + 2] = fz[i];
  }
}

unsigned char* g_scratch_ptr[RD_NOALLOC_MAX_DEVICES] = {};
std::mutex g_scratch_mu;

// Device address of g_noalloc_scratch on `device` (resolved once per device,
// with that device current).
int scratch_for_device(int device, unsigned char** out) {
  if (device < 0 || device >= RD_NOALLOC_MAX_DEVICES) return rd_set_error(RD_ERR_INVALID, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[device]) {
    int prev = 0;
    cudaError_t e = cudaGetDevice(&prev);
    if (e != cudaSuccess) return rd_set_error(RD_ERR_CUDA, cudaGetErrorString(e));
    if (prev != device && (e = cudaSetDevice(device)) != cudaSuccess)
      return rd_set_error(RD_ERR_CUDA, cudaGetErrorString(e));
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (prev != device) cudaSetDevice(prev);
    if (e != cudaSuccess || !p)
      return rd_set_error(RD_ERR_CUDA, (std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e)).c_str());
    g_scratch_ptr[device] = (unsigned char*)p;
  }
  *out = g_scratch_ptr[device];
  return RD_OK;
}

}  // namespace

// Set-up of the no-allocation path on `device` for an engine of precision
// `prec` (called by rd_engine_create with that device current): loads the
// module of this file (array and kernels) and the kernels the call launches,
// and resolves the array's device address.
int rd_noalloc_prepare(int device, int prec) {
  unsigned char* s = nullptr;
  int rc = scratch_for_device(device, &s);
  if (rc) return rc;
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, k_na_begin);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, k_na_end);
  if (e == cudaSuccess) e = rd_preload_field_points(prec);
  if (e == cudaSuccess) e = rd_preload_plan();
  if (e != cudaSuccess) return rd_set_error(RD_ERR_CUDA, cudaGetErrorString(e));
  return RD_OK;
}

// Makes `device` current for the lifetime of the object and restores the
// caller's device afterwards.
struct DeviceScope {
  int prev = -1;
  cudaError_t err = cudaSuccess;
  explicit DeviceScope(int device) {
    err = cudaGetDevice(&prev);
    if (err == cudaSuccess && prev != device) err = cudaSetDevice(device);
    else if (err == cudaSuccess) prev = -1;   // nothing to restore
  }
  ~DeviceScope() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

extern "C" int rd_field_at_noalloc(rd_engine* e, int diode, int M, const double* pos3m_dev,
                                   double* field3m_dev) {
  if (!e) return rd_set_error(RD_ERR_INVALID, "null engine");
  if (M < 0 || M > RD_NOALLOC_MAX_POINTS)
    return rd_set_error(RD_ERR_INVALID, "rd_field_at_noalloc: M must be in [0, 65536] (the size of its static scratch)");
  if (M > 0 && (!pos3m_dev || !field3m_dev)) return rd_set_error(RD_ERR_INVALID, "null device pointer");
  const DiodeParams* P;
  const DiodeDyn* Dy;
  Pool pool;
  int geom, prec, grid, device;
  double kscale;
  cudaStream_t st;
  int rc = rd_engine_view(e, diode, &P, &Dy, &pool, &geom, &prec, &grid, &kscale, &st, &device);
  if (rc) return rc;
  if (M == 0) return RD_OK;
  DeviceScope scope(device);   // the engine's stream and the scratch address belong to its device
  if (scope.err != cudaSuccess) return rd_set_error(RD_ERR_CUDA, cudaGetErrorString(scope.err));
  unsigned char* s = nullptr;
  if ((rc = scratch_for_device(device, &s))) return rc;
  PlanEntry* plan = (PlanEntry*)(s + NA_OFF_PLAN);
  PlanHeader* ph = (PlanHeader*)(s + NA_OFF_HDR);
  int* ints = (int*)(s + NA_OFF_INTS);
  double* px = (double*)(s + NA_OFF_PTS);
  double* fx = (double*)(s + NA_OFF_FLD);
  double* partial = (double*)(s + NA_OFF_PART);
  int* tickets = (int*)(s + NA_OFF_TICK);
  // the particle packs must be current (kernels only, no allocation)
  if ((rc = rd_engine_repack(e))) return rc;
  k_na_begin<<<64, 256, 0, st>>>(ints, M, tickets, NA_MAX_ITEMS, pos3m_dev, px,
                                 px + RD_NOALLOC_MAX_POINTS, px + 2 * RD_NOALLOC_MAX_POINTS);
  cudaError_t ce = cudaGetLastError();
  if (ce == cudaSuccess)
    ce = rd_launch_plan(st, P, Dy, 1, PM_FIELD, rd_engine_chunk_rule(e), NA_MAX_ITEMS, ints, plan, ph);
  PointSet pts{px, px + RD_NOALLOC_MAX_POINTS, px + 2 * RD_NOALLOC_MAX_POINTS,
               fx, fx + RD_NOALLOC_MAX_POINTS, fx + 2 * RD_NOALLOC_MAX_POINTS, ints + 1};
  if (ce == cudaSuccess)
    ce = rd_launch_field_points(prec, geom, grid, st, P, pool, plan, ph, pts, partial, tickets, kscale);
  if (ce == cudaSuccess) {
    k_na_end<<<64, 256, 0, st>>>(M, fx, fx + RD_NOALLOC_MAX_POINTS, fx + 2 * RD_NOALLOC_MAX_POINTS,
                                 field3m_dev);
    ce = cudaGetLastError();
  }
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
  if (ce != cudaSuccess) return rd_set_error(RD_ERR_CUDA, cudaGetErrorString(ce));
  return RD_OK;
}
