// Device-driven barotropic step (sm_103a).
//
// One call of cmm_bve_step enqueues the whole main-loop body of
// euler_simulation_sphere_remapping (cmm_s2/core/spherical_simulations.py:
// 263-294): the RK4 map update, the assembly of the current map, the
// composition of the MWSS sample points through the submap stack and the
// current map, the vorticity there, its inversion to velocity jets and their
// assembly into the oldest velocity slot, then the driver's bookkeeping
// (remap into the stack, velocity-slot rotation, times and stage weights).
// Everything that changes from step to step lives in a device-resident
// BveState that the kernels read, and the bookkeeping runs on the device,
// so the launches of every step are identical: a CUDA graph captured from
// one call replays all later steps, and the graphs of many runs can be
// captured into one (an ensemble advanced by one graph launch per step).
//
// The stage weights are recomputed on the device with the operations and
// rounding of the host's time_weights (no contraction), so a device-driven
// run is bit-identical to the same run driven from the host.
#include <cuda_runtime.h>

#include <new>
#include <vector>

#include "cmm_internal.h"
#include "device_common.cuh"

namespace cmm {

namespace {

// RK4 stage times t + dt, t + dt/2, t + 0.5 dt, t and their quadratic
// Lagrange weights on the nodes ts0, ts0 + dt, ts0 + 2 dt, evaluated
// exactly as time_weights / stage_weights do on the host.
__device__ void rk4_weights(double ts0, double t, double dt, TimeWeights* tw) {
  const double times[4] = {__dadd_rn(t, dt), __dadd_rn(t, __ddiv_rn(dt, 2.0)),
                           __dadd_rn(t, __dmul_rn(0.5, dt)), t};
  const double t0 = ts0, t1 = __dadd_rn(ts0, dt), t2 = __dadd_rn(ts0, __dmul_rn(2.0, dt));
  const double dd2 = __dmul_rn(__dmul_rn(2.0, dt), dt), ndd = __dmul_rn(-dt, dt);
  for (int s = 0; s < 4; ++s) {
    const double t_ = times[s];
    tw->w[s][0] = __ddiv_rn(__dmul_rn(__dsub_rn(t_, t1), __dsub_rn(t_, t2)), dd2);
    tw->w[s][1] = __ddiv_rn(__dmul_rn(__dsub_rn(t_, t0), __dsub_rn(t_, t2)), ndd);
    tw->w[s][2] = __ddiv_rn(__dmul_rn(__dsub_rn(t_, t0), __dsub_rn(t_, t1)), dd2);
  }
}

// Remap step of the driver (spherical_simulations.py:284-294) when the
// step about to complete (count + 1) is in ns = {n_maps, 2 n_maps, ...} u
// {Nt}: index of its stack slot, else -1.
__device__ __forceinline__ int remap_slot(int c, int n_maps, int Nt) {
  if (c == Nt) return (Nt - 1) / n_maps;
  if (c < Nt && c % n_maps == 0) return c / n_maps - 1;
  return -1;
}

// Copies of the remap: current map -> stack slot, its jets -> jets slot
// (optional), jets <- identity jets.  A no-op on steps without a remap.
__global__ void bve_remap_kernel(const BveState* __restrict__ st, int n_maps, int Nt,
                                 const double* __restrict__ cur, double* const* __restrict__ table,
                                 int64_t nrec, double* __restrict__ jets,
                                 double* const* __restrict__ jtable, const double* __restrict__ id_jets,
                                 int64_t njets) {
  const int slot = remap_slot(st->count + 1, n_maps, Nt);
  if (slot < 0) return;
  double* dst = table[slot];
  double* jdst = jtable ? jtable[slot] : nullptr;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nrec; i += stride) dst[i] = cur[i];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < njets; i += stride) {
    if (jdst) jdst[i] = jets[i];
    jets[i] = id_jets[i];
  }
}

// Driver bookkeeping at the end of a step (spherical_simulations.py:
// 273-294): count, remap flags, velocity slots (the slot just written
// becomes the newest), ts0 and the next step's stage weights.
__global__ void bve_advance_kernel(BveState* st, int n_maps, int Nt) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int c = st->count + 1;
  const int slot = remap_slot(c, n_maps, Nt);
  st->count = c;
  st->identity = slot >= 0 ? 1 : 0;
  if (slot >= 0) st->nc = slot + 1;
  double* v0 = st->vel[0];
  st->vel[0] = st->vel[1];
  st->vel[1] = st->vel[2];
  st->vel[2] = v0;
  st->ts0 = __dadd_rn(st->ts0, st->step);
  st->k += 1;
  rk4_weights(st->ts0, __dmul_rn((double)st->k, st->step), st->step, &st->tw);
}

// Initial weights from the host-supplied state.
__global__ void bve_init_kernel(BveState* st) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  rk4_weights(st->ts0, __dmul_rn((double)st->k, st->step), st->step, &st->tw);
}

int check(const char* what) {
  note_launch();
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? CMM_OK : cuda_fail(e, what);
}

}  // namespace
}  // namespace cmm

struct cmm_bve {
  cmm_bve_desc d;
  cmm::DeviceBuffer state, table, jtable, ftable;
  int64_t nrec = 0, njets = 0, nsample = 0;
};

namespace cmm {

int bve_create(const cmm_bve_desc* d, cmm_bve** out) {
  if (!d || !out || !d->mesh || !d->velmesh || !d->sht || d->mesh->view.kind != kIcosahedral ||
      d->velmesh->view.kind != kLatLon || sht_L(d->sht) != d->velmesh->view.L || !d->s_pts ||
      !d->tan || !d->id_jets || !d->sample_pts || !d->jets || !d->coeffs_cur || !d->work || !d->X ||
      !d->omega || !d->vel_jets || !d->vel[0] || !d->vel[1] || !d->vel[2] || d->n_stack < 1 ||
      !d->stack || d->n_maps < 1 || d->Nt < 3 || d->nparams < 0 || d->nparams > 12 ||
      d->vort_kind < 0 || d->vort_kind > 6 || (d->sh && (d->lmax < 0 || d->lmax > kShTableMax)) || d->nc < 0 ||
      d->nc > d->n_stack || d->n_stack > CMM_MAX_SUBMAPS - 1 || !(d->tspan_step > 0.0)) {
    set_last_error("cmm_bve_create: bad descriptor");
    return CMM_ERR_ARG;
  }
  // every remap slot the run can reach must exist
  if ((d->Nt - 1) / d->n_maps + 1 > d->n_stack) {
    set_last_error("cmm_bve_create: n_stack smaller than the number of remaps of the run");
    return CMM_ERR_ARG;
  }
  for (int k = 0; k < d->n_stack; ++k)
    if (!d->stack[k] || (d->stack_forms && !d->stack_forms[k])) {
      set_last_error("cmm_bve_create: null stack slot");
      return CMM_ERR_ARG;
    }
  cmm_bve* b = new (std::nothrow) cmm_bve();
  if (!b) {
    set_last_error("cmm_bve_create: out of host memory");
    return CMM_ERR_NOMEM;
  }
  b->d = *d;
  b->d.stack = nullptr;
  b->d.stack_jets = nullptr;
  b->d.stack_forms = nullptr;
  const int L = d->velmesh->view.L;
  b->nrec = (int64_t)d->mesh->view.nt * kCoeffStride3;
  b->njets = 12LL * d->mesh->view.nv;
  b->nsample = (int64_t)(L + 1) * 2 * L;
  BveState h{};
  for (int k = 0; k < 3; ++k) h.vel[k] = d->vel[k];
  h.ts0 = d->ts0;
  h.step = d->tspan_step;
  h.k = d->k;
  h.count = d->count;
  h.nc = d->nc;
  h.identity = d->identity;
  int rc;
  if ((rc = b->state.upload(&h, sizeof(h))) ||
      (rc = b->table.upload(d->stack, sizeof(double*) * d->n_stack)) ||
      (d->stack_jets && (rc = b->jtable.upload(d->stack_jets, sizeof(double*) * d->n_stack))) ||
      (d->stack_forms && (rc = b->ftable.upload(d->stack_forms, sizeof(double*) * d->n_stack)))) {
    delete b;
    return rc;
  }
  bve_init_kernel<<<1, 1>>>((BveState*)b->state.p);
  if ((rc = check("bve_init_kernel"))) {
    delete b;
    return rc;
  }
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    delete b;
    return cuda_fail(e, "cmm_bve_create");
  }
  *out = b;
  return CMM_OK;
}

int bve_destroy(cmm_bve* b) {
  delete b;
  return CMM_OK;
}

// The step's first half: map update and assembly, the sample points
// through the stack, the vorticity there; then (batched) the forward
// transform up to the member's data tiles, or (alone) the whole velocity
// inversion.
static int step_first(cmm_bve* b, cudaStream_t s, bool batched) {
  const cmm_bve_desc& d = b->d;
  const MeshView& mesh = d.mesh->view;
  const MeshView& vm = d.velmesh->view;
  const BveState* st = (const BveState*)b->state.p;
  int rc;
  // map update (RK4 through the three velocity levels) and its assembly
  if ((rc = launch_advect_points(mesh, vm, VelPtrs{}, 3, TimeWeights{}, CMM_RK4, d.tspan_step, d.s_pts,
                                 d.work, s, st)))
    return rc;
  if ((rc = launch_project_jets(mesh, d.coeffs_cur, d.work, d.work + 3 * (int64_t)mesh.nv, d.tan,
                                d.eps, d.jets, s, st)))
    return rc;
  if ((rc = launch_assemble(mesh, d.jets, 3, d.coeffs_cur, s))) return rc;
  // sample points through stack and current map, vorticity, velocity
  if ((rc = launch_compose_dev(mesh, (const double* const*)b->table.p, st, d.coeffs_cur, d.sample_pts,
                               b->nsample, d.X, s, (const double* const*)b->ftable.p)))
    return rc;
  if ((rc = launch_vorticity(d.vort_kind, d.vort_params, d.nparams, d.sh, d.lmax, vm, d.spline,
                             d.rot_rate, d.X, b->nsample, 2 * vm.L,
                             (const double*)d.velmesh->cos_theta.p, d.omega, s)))
    return rc;
  if (batched) return sht_velocity_pre(d.sht, d.omega, s);
  return sht_velocity(d.sht, d.velmesh, d.omega, nullptr, d.vel_jets, s);
}

// The second half: the velocity levels, remap and bookkeeping.
static int step_second(cmm_bve* b, cudaStream_t s) {
  const cmm_bve_desc& d = b->d;
  const MeshView& mesh = d.mesh->view;
  const MeshView& vm = d.velmesh->view;
  const BveState* st = (const BveState*)b->state.p;
  int rc;
  // FP32 records from the split form's FP32 jets (the same values as the
  // double jets, without the conversions)
  const float* jf = vm.rec32 ? sht_jets_f32(d.sht) : nullptr;
  if ((rc = jf ? launch_assemble_f32_jets(vm, jf, s, st) : launch_assemble(vm, d.vel_jets, 3, nullptr, s, st)))
    return rc;
  // bookkeeping
  const int64_t nmax = b->nrec > b->njets ? b->nrec : b->njets;
  bve_remap_kernel<<<dev::grid_for(nmax, 256), 256, 0, s>>>(st, d.n_maps, d.Nt, d.coeffs_cur,
                                                       (double* const*)b->table.p, b->nrec, d.jets,
                                                       (double* const*)b->jtable.p, d.id_jets, b->njets);
  if ((rc = check("bve_remap_kernel"))) return rc;
  if (b->ftable.p &&
      (rc = launch_remap_forms(mesh, st, d.n_maps, d.Nt, (const double* const*)b->table.p,
                               (double* const*)b->ftable.p, s)))
    return rc;
  bve_advance_kernel<<<1, 32, 0, s>>>((BveState*)b->state.p, d.n_maps, d.Nt);
  return check("bve_advance_kernel");
}

int bve_step(cmm_bve* b, cudaStream_t s) {
  int rc = step_first(b, s, false);
  return rc ? rc : step_second(b, s);
}

int bve_step_pre(cmm_bve* b, cudaStream_t s) { return step_first(b, s, true); }

int bve_step_post(cmm_bve* b, cudaStream_t s) {
  const cmm_bve_desc& d = b->d;
  int rc = sht_velocity_post(d.sht, d.velmesh, d.vel_jets, s);
  return rc ? rc : step_second(b, s);
}

int bve_state(cmm_bve* b, cudaStream_t s, int* count, int* nc, int* identity) {
  BveState h;
  cudaError_t e = cudaMemcpyAsync(&h, b->state.p, sizeof(h), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "cmm_bve_state");
  if (count) *count = h.count;
  if (nc) *nc = h.nc;
  if (identity) *identity = h.identity;
  return CMM_OK;
}

}  // namespace cmm
