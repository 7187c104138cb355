// extern "C" entry points of libcmmgpu.so: argument checks, then the
// launchers of the kernel translation units.
#include <new>

#include "cmm_internal.h"

using namespace cmm;

namespace {
int arg_error(const char* msg) {
  set_last_error(msg);
  return CMM_ERR_ARG;
}
}  // namespace

extern "C" {

const char* cmm_last_error(void) { return last_error(); }

int cmm_version(void) { return 1; }

long long cmm_launch_count(void) { return launch_count(); }

int cmm_mesh_create(const double* verts, int nv, const int32_t* tris, int nt, int level,
                    cmm_mesh** out) {
  if (!verts || !tris || !out) return arg_error("cmm_mesh_create: null pointer");
  *out = nullptr;
  cmm_mesh* m = new (std::nothrow) cmm_mesh();
  if (!m) {
    set_last_error("cmm_mesh_create: out of host memory");
    return CMM_ERR_NOMEM;
  }
  int rc = CMM_OK;
  HostMesh hm;
  if (!rc) rc = build_host(verts, nv, tris, nt, level, &hm);
  if (!rc) rc = upload_mesh(hm, m);
  if (rc) {
    delete m;
    return rc;
  }
  *out = m;
  return CMM_OK;
}

int cmm_mesh_check(const double* verts, int nv, const int32_t* tris, int nt, int level,
                   int32_t* leaf_row) {
  if (!verts || !tris) return arg_error("cmm_mesh_check: null pointer");
  HostMesh hm;
  int rc = build_host(verts, nv, tris, nt, level, &hm);
  if (!rc && leaf_row)
    for (int i = 0; i < nt; ++i) leaf_row[i] = hm.leaf_row[i];
  return rc;
}

int cmm_mesh_destroy(cmm_mesh* mesh) {
  delete mesh;
  return CMM_OK;
}

int cmm_mesh_status(cmm_mesh* mesh, void* stream, int* flags, int clear) {
  if (!mesh || !flags) return arg_error("cmm_mesh_status: null pointer");
  cudaStream_t s = (cudaStream_t)stream;
  int h = 0;
  cudaError_t e = cudaMemcpyAsync(&h, mesh->view.status, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "cmm_mesh_status");
  *flags = h;
  if (clear) {
    e = cudaMemsetAsync(mesh->view.status, 0, sizeof(int), s);
    if (e != cudaSuccess) return cuda_fail(e, "cmm_mesh_status(clear)");
  }
  return CMM_OK;
}

int cmm_coeff_stride(int ncomp) {
  return ncomp == 3 ? kCoeffStride3 : (ncomp == 1 ? kCoeffStride1 : -1);
}

int cmm_locate(const cmm_mesh* mesh, const double* q, int64_t n, int32_t* tri, double* bcc,
               void* stream) {
  if (!mesh || n < 0 || (n > 0 && (!q || !tri))) return arg_error("cmm_locate: bad argument");
  if (mesh->view.kind == kLatLon)
    return launch_latlon_locate(mesh->view, q, n, tri, bcc, (cudaStream_t)stream);
  return launch_locate(mesh->view, q, n, tri, bcc, (cudaStream_t)stream);
}

int cmm_velmesh_create(int L, const double* theta, const double* phi, const double* grid,
                       const double* verts, cmm_mesh** out) {
  if (!theta || !phi || !grid || !verts || !out) return arg_error("cmm_velmesh_create: null pointer");
  *out = nullptr;
  cmm_mesh* m = new (std::nothrow) cmm_mesh();
  if (!m) {
    set_last_error("cmm_velmesh_create: out of host memory");
    return CMM_ERR_NOMEM;
  }
  int rc = build_latlon(L, theta, phi, grid, verts, m);
  if (rc) {
    delete m;
    return rc;
  }
  *out = m;
  return CMM_OK;
}

namespace {
int vel_args(const cmm_mesh* vm, const double* const* vc, int nvs, VelPtrs* out, const char* who) {
  if (!vm || vm->view.kind != kLatLon) {
    set_last_error(std::string(who) + ": velocity mesh expected");
    return CMM_ERR_ARG;
  }
  if (nvs < 1 || nvs > 3 || !vc) {
    set_last_error(std::string(who) + ": nvs must be 1..3");
    return CMM_ERR_ARG;
  }
  *out = VelPtrs{};
  for (int l = 0; l < nvs; ++l) {
    if (!vc[l]) {
      set_last_error(std::string(who) + ": null velocity coefficients");
      return CMM_ERR_ARG;
    }
    out->p[l] = vc[l];
  }
  return CMM_OK;
}

int stage_weights(int nvs, double ts0, int scheme, double t, double dt, TimeWeights* tw) {
  // stage times of each integrator (cmm_s2/core/evolution_functions.py:19-80)
  double times[4];
  const int nt = stage_times(scheme, t, dt, times);
  if (nt == 0) return arg_error("unknown integration scheme");
  *tw = time_weights(nvs, ts0, dt, times, nt);
  return CMM_OK;
}
}  // namespace

int cmm_velocity_eval(const cmm_mesh* velmesh, const double* const* vel_coeffs, int nvs,
                      double ts0, double t, double dt, const double* x, int64_t n, double* out,
                      void* stream) {
  VelPtrs vc;
  int rc = vel_args(velmesh, vel_coeffs, nvs, &vc, "cmm_velocity_eval");
  if (rc) return rc;
  if (n < 0 || (n > 0 && (!x || !out))) return arg_error("cmm_velocity_eval: bad argument");
  TimeWeights tw = time_weights(nvs, ts0, dt, &t, 1);
  return launch_velocity_eval(velmesh->view, vc, nvs, tw, x, n, out, (cudaStream_t)stream);
}

int cmm_integrate(const cmm_mesh* velmesh, const double* const* vel_coeffs, int nvs, double ts0,
                  int scheme, double t, double dt, const double* x, int64_t n, double* out,
                  void* stream) {
  VelPtrs vc;
  int rc = vel_args(velmesh, vel_coeffs, nvs, &vc, "cmm_integrate");
  if (rc) return rc;
  if (n < 0 || (n > 0 && (!x || !out))) return arg_error("cmm_integrate: bad argument");
  TimeWeights tw;
  if ((rc = stage_weights(nvs, ts0, scheme, t, dt, &tw))) return rc;
  return launch_integrate(velmesh->view, vc, nvs, tw, scheme, dt, x, n, out, (cudaStream_t)stream);
}

int cmm_vorticity_eval(const cmm_mesh* velmesh, int kind, const double* params, int nparams,
                       const double* sh, int lmax, const double* spline, double rot_rate,
                       const double* X, double* omega, void* stream) {
  if (!velmesh || velmesh->view.kind != kLatLon) return arg_error("cmm_vorticity_eval: velocity mesh expected");
  if (!X || !omega || (nparams > 0 && !params) || nparams > 12 || kind < 0 || kind > 7 ||
      (sh && (lmax < 0 || lmax > kShTableMax)))
    return arg_error("cmm_vorticity_eval: bad argument (series degree lmax must be in [0, 128])");
  const int L = velmesh->view.L;
  const int64_t Q = (int64_t)(L + 1) * 2 * L;
  return launch_vorticity(kind, params, nparams, sh, lmax, velmesh->view, spline, rot_rate, X, Q,
                          2 * L, (const double*)velmesh->cos_theta.p, omega, (cudaStream_t)stream);
}

int cmm_sht_scalar_jets(cmm_sht* plan, const cmm_mesh* velmesh, const double* alm, double* jets,
                        void* stream) {
  if (!plan || !velmesh || !alm || !jets) return arg_error("cmm_sht_scalar_jets: null pointer");
  if (velmesh->view.kind != kLatLon || velmesh->view.L != sht_L(plan))
    return arg_error("cmm_sht_scalar_jets: velocity mesh of the plan's band-limit expected");
  return sht_scalar_jets(plan, velmesh, (const double2*)alm, jets, (cudaStream_t)stream);
}

int cmm_advect_project_noalloc(const cmm_mesh* mesh, const cmm_mesh* velmesh,
                               const double* const* vel_coeffs, int nvs, double ts0, int scheme,
                               double t, double dt, const double* s_pts, const double* tan,
                               const double* prev_coeffs, double eps, double* jets, void* stream) {
  if (!mesh || mesh->view.kind != kIcosahedral)
    return arg_error("cmm_advect_project_noalloc: map mesh expected");
  VelPtrs vc;
  int rc = vel_args(velmesh, vel_coeffs, nvs, &vc, "cmm_advect_project_noalloc");
  if (rc) return rc;
  if (!s_pts || !tan || !jets) return arg_error("cmm_advect_project_noalloc: null pointer");
  TimeWeights tw;
  if ((rc = stage_weights(nvs, ts0, scheme, t, dt, &tw))) return rc;
  return advect_project_noalloc(mesh->view, velmesh->view, vc, nvs, tw, scheme, dt, s_pts, tan,
                                prev_coeffs, eps, jets, (cudaStream_t)stream);
}

int cmm_sht_create(int L, cmm_sht** out) {
  if (!out) return arg_error("cmm_sht_create: null pointer");
  *out = nullptr;
  return sht_create(L, out);
}

int cmm_sht_destroy(cmm_sht* plan) { return plan ? sht_destroy(plan) : CMM_OK; }

int cmm_sht_set_precision(cmm_sht* plan, int mode) {
  if (!plan) return arg_error("cmm_sht_set_precision: null pointer");
  return sht_set_precision(plan, mode);
}

int cmm_sht_timeout_selftest(cmm_sht* plan, long long polls, void* stream) {
  if (!plan || polls < 1 || polls > (1LL << 20))
    return arg_error("cmm_sht_timeout_selftest: polls must be in [1, 2^20]");
  return tc_wait_timeout_probe(polls, sht_status_word(plan), (cudaStream_t)stream);
}

int cmm_sht_set_schedule(cmm_sht* plan, int schedule) {
  if (!plan) return arg_error("cmm_sht_set_schedule: null pointer");
  return sht_set_schedule(plan, schedule);
}

int cmm_sht_set_tables(cmm_sht* plan, int mode) {
  if (!plan) return arg_error("cmm_sht_set_tables: null pointer");
  return sht_set_tables(plan, mode);
}

int cmm_velmesh_set_records(cmm_mesh* velmesh, int precision) {
  if (!velmesh || velmesh->view.kind != kLatLon) return arg_error("cmm_velmesh_set_records: velocity mesh expected");
  if (precision != CMM_REC_FP64 && precision != CMM_REC_FP32 && precision != CMM_REC_MIXED)
    return arg_error("cmm_velmesh_set_records: unknown precision");
  if (precision != CMM_REC_FP64 && !velmesh->view.tri_asm_f) {
    int rc = make_asm_f32(velmesh);
    if (rc) return rc;
  }
  velmesh->view.rec32 = precision != CMM_REC_FP64 ? 1 : 0;
  velmesh->view.field32 = precision == CMM_REC_MIXED ? 1 : 0;
  return CMM_OK;
}

int cmm_mesh_set_block(cmm_mesh* mesh, int kernel, int threads) {
  if (!mesh || kernel < 0 || kernel > 3 || threads < 0 || threads > 256 || threads % 32 != 0)
    return arg_error("cmm_mesh_set_block: bad argument");
  mesh->view.block[kernel] = threads;
  return CMM_OK;
}

int cmm_mesh_set_variant(cmm_mesh* mesh, int knob, int value) {
  const bool ok = mesh && ((knob == CMM_VARIANT_COMPOSE_JAC && (value == 0 || (value >= 2 && value <= 4))) ||
                           (knob == CMM_VARIANT_COMPOSE && (value == 0 || value == 4 || value == 6)));
  if (!ok) return arg_error("cmm_mesh_set_variant: bad argument");
  mesh->view.variant[knob] = value;
  return CMM_OK;
}

int cmm_bve_create(const cmm_bve_desc* desc, cmm_bve** out) { return bve_create(desc, out); }

int cmm_bve_destroy(cmm_bve* bve) { return bve_destroy(bve); }

int cmm_bve_step(cmm_bve* bve, void* stream) {
  if (!bve) return arg_error("cmm_bve_step: null handle");
  return bve_step(bve, (cudaStream_t)stream);
}

int cmm_bve_step_pre(cmm_bve* bve, void* stream) {
  if (!bve) return arg_error("cmm_bve_step_pre: null handle");
  return bve_step_pre(bve, (cudaStream_t)stream);
}

int cmm_bve_step_post(cmm_bve* bve, void* stream) {
  if (!bve) return arg_error("cmm_bve_step_post: null handle");
  return bve_step_post(bve, (cudaStream_t)stream);
}

int cmm_bve_state(cmm_bve* bve, void* stream, int* count, int* nc, int* identity) {
  if (!bve) return arg_error("cmm_bve_state: null handle");
  return bve_state(bve, (cudaStream_t)stream, count, nc, identity);
}

int cmm_assemble_bwd(const cmm_mesh* mesh, const double* grad_coeffs, double* grad_jets, void* stream) {
  if (!mesh || !grad_coeffs || !grad_jets) return arg_error("cmm_assemble_bwd: null pointer");
  if (mesh->view.rec32) return arg_error("cmm_assemble_bwd: FP64 records expected");
  return launch_assemble_bwd(mesh->view, grad_coeffs, grad_jets, (cudaStream_t)stream);
}

int cmm_compose_bwd(const cmm_mesh* mesh, const double* const* coeffs, int S, const double* q, int64_t n,
                    const double* grad_out, double* const* grad_coeffs, double* grad_q, double* work,
                    void* stream) {
  if (!mesh || S < 1 || S > kAdjMaxSubmaps || !coeffs || !grad_coeffs || n < 0 ||
      (n > 0 && (!q || !grad_out || !work)))
    return arg_error("cmm_compose_bwd: bad argument");
  for (int k = 0; k < S; ++k)
    if (!coeffs[k] || !grad_coeffs[k]) return arg_error("cmm_compose_bwd: null submap");
  return launch_compose_bwd(mesh->view, coeffs, grad_coeffs, S, q, n, grad_out, grad_q, work,
                            (cudaStream_t)stream);
}

int cmm_advect_project_bwd(const cmm_mesh* mesh, const cmm_mesh* velmesh, const double* const* vel_coeffs,
                           int nvs, double ts0, int scheme, double t, double dt, const double* s_pts,
                           const double* tan, const double* prev_coeffs, double eps, const double* grad_jets,
                           double* const* grad_vel, double* grad_prev, double* work, void* stream) {
  if (!mesh || mesh->view.kind != kIcosahedral) return arg_error("cmm_advect_project_bwd: map mesh expected");
  VelPtrs vc;
  int rc = vel_args(velmesh, vel_coeffs, nvs, &vc, "cmm_advect_project_bwd");
  if (rc) return rc;
  if (velmesh->view.rec32) return arg_error("cmm_advect_project_bwd: FP64 velocity records expected");
  if (scheme != CMM_EULER && scheme != CMM_IMPROVED_EULER && scheme != CMM_RK4)
    return arg_error("cmm_advect_project_bwd: scheme 0, 1 or 2 expected");
  if (!s_pts || !tan || !grad_jets || !grad_vel || !work) return arg_error("cmm_advect_project_bwd: null pointer");
  for (int l = 0; l < nvs; ++l)
    if (!grad_vel[l]) return arg_error("cmm_advect_project_bwd: null velocity cotangent");
  TimeWeights tw;
  if ((rc = stage_weights(nvs, ts0, scheme, t, dt, &tw))) return rc;
  return launch_advect_project_bwd(mesh->view, velmesh->view, vel_coeffs, grad_vel, nvs, tw, scheme, dt, s_pts,
                                   tan, prev_coeffs, grad_prev, eps, grad_jets, work, (cudaStream_t)stream);
}

int cmm_vorticity_bwd(const cmm_mesh* velmesh, const double* dsh, int lmax, double rot_rate,
                      const double* X, const double* grad_omega, double* grad_X, double* grad_sh,
                      void* stream) {
  if (!velmesh || velmesh->view.kind != kLatLon || !X || !grad_omega)
    return arg_error("cmm_vorticity_bwd: bad argument");
  const int L = velmesh->view.L;
  const int64_t Q = (int64_t)(L + 1) * 2 * L;
  return launch_vorticity_bwd(velmesh->view, dsh, lmax, rot_rate, X, Q, grad_omega, grad_X, grad_sh,
                              (cudaStream_t)stream);
}

int cmm_sht_velocity_bwd(cmm_sht* plan, const cmm_mesh* velmesh, const double* grad_jets, double* grad_omega,
                         void* stream) {
  if (!plan || !velmesh || velmesh->view.kind != kLatLon || velmesh->view.L != sht_L(plan) || !grad_jets ||
      !grad_omega)
    return arg_error("cmm_sht_velocity_bwd: bad argument");
  return sht_velocity_bwd(plan, velmesh, grad_jets, grad_omega, (cudaStream_t)stream);
}

int cmm_sht_power(cmm_sht* plan, const double* alm, double* power, void* stream) {
  if (!plan || !alm || !power) return arg_error("cmm_sht_power: null pointer");
  return sht_power(plan, (const double2*)alm, power, (cudaStream_t)stream);
}

int cmm_sht_share_tables(cmm_sht* plan, cmm_sht* src) {
  if (!plan || !src) return arg_error("cmm_sht_share_tables: null plan");
  return sht_share_tables(plan, src);
}

int cmm_sht_trim(cmm_sht* plan) {
  if (!plan) return arg_error("cmm_sht_trim: null plan");
  return sht_trim(plan);
}

int cmm_sht_batch_create(cmm_sht* const* plans, int n, cmm_sht_batch** out) {
  return sht_batch_create(plans, n, out);
}

int cmm_sht_batch_destroy(cmm_sht_batch* batch) { return sht_batch_destroy(batch); }

int cmm_sht_batch_analysis(cmm_sht_batch* batch, void* stream) {
  if (!batch) return arg_error("cmm_sht_batch_analysis: null batch");
  return sht_batch_analysis(batch, nullptr, (cudaStream_t)stream);
}

int cmm_sht_batch_forward(cmm_sht_batch* batch, const double* const* samples, double* const* alm,
                          void* stream) {
  if (!batch || !samples || !alm) return arg_error("cmm_sht_batch_forward: null pointer");
  for (int b = 0; b < sht_batch_size(batch); ++b)
    if (!samples[b] || !alm[b]) return arg_error("cmm_sht_batch_forward: null member pointer");
  return sht_batch_forward(batch, samples, (double2* const*)alm, (cudaStream_t)stream);
}

int cmm_sht_status(cmm_sht* plan, void* stream, int* flags, int clear) {
  if (!plan || !flags) return arg_error("cmm_sht_status: null pointer");
  return sht_status(plan, (cudaStream_t)stream, flags, clear);
}

int cmm_sht_forward(cmm_sht* plan, const double* samples, double* alm, void* stream) {
  if (!plan || !samples || !alm) return arg_error("cmm_sht_forward: null pointer");
  return sht_forward(plan, samples, (double2*)alm, (cudaStream_t)stream);
}

int cmm_sht_inverse(cmm_sht* plan, const double* alm, int nf, double* samples, void* stream) {
  if (!plan || !alm || !samples || (nf != 1 && nf != 12))
    return arg_error("cmm_sht_inverse: bad argument (nf must be 1 or 12)");
  return sht_inverse(plan, (const double2*)alm, nf, samples, (cudaStream_t)stream);
}

int cmm_sht_velocity(cmm_sht* plan, const cmm_mesh* velmesh, const double* omega, double* psi,
                     double* vel_jets, void* stream) {
  if (!plan || !velmesh || (!omega && !psi) || !vel_jets)
    return arg_error("cmm_sht_velocity: null pointer");
  if (velmesh->view.kind != kLatLon || velmesh->view.L != sht_L(plan))
    return arg_error("cmm_sht_velocity: velocity mesh of the plan's band-limit expected");
  return sht_velocity(plan, velmesh, omega, (double2*)psi, vel_jets, (cudaStream_t)stream);
}

int64_t cmm_advect_workspace(const cmm_mesh* mesh) {
  return mesh ? 15LL * mesh->view.nv : -1;
}

int cmm_advect_project(const cmm_mesh* mesh, const cmm_mesh* velmesh,
                       const double* const* vel_coeffs, int nvs, double ts0, int scheme, double t,
                       double dt, const double* s_pts, const double* tan,
                       const double* prev_coeffs, double eps, double* jets, double* work,
                       void* stream) {
  if (!mesh || mesh->view.kind != kIcosahedral) return arg_error("cmm_advect_project: map mesh expected");
  VelPtrs vc;
  int rc = vel_args(velmesh, vel_coeffs, nvs, &vc, "cmm_advect_project");
  if (rc) return rc;
  if (!s_pts || !tan || !jets || !work) return arg_error("cmm_advect_project: null pointer");
  TimeWeights tw;
  if ((rc = stage_weights(nvs, ts0, scheme, t, dt, &tw))) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  if ((rc = launch_advect_points(mesh->view, velmesh->view, vc, nvs, tw, scheme, dt, s_pts, work, s)))
    return rc;
  const int64_t nv = mesh->view.nv;
  return launch_project_jets(mesh->view, prev_coeffs, work, work + 3 * nv, tan, eps, jets, s);
}

int cmm_assemble(const cmm_mesh* mesh, const double* jets, int ncomp, double* coeffs,
                 void* stream) {
  if (!mesh || !jets || !coeffs || (ncomp != 1 && ncomp != 3))
    return arg_error("cmm_assemble: bad argument");
  return launch_assemble(mesh->view, jets, ncomp, coeffs, (cudaStream_t)stream);
}

int cmm_compose(const cmm_mesh* mesh, const double* const* coeffs, int S, const double* q,
                int64_t n, double* out, int32_t* tri, int32_t* tri_all, double* jac,
                void* stream) {
  if (!mesh || S < 1 || S > CMM_MAX_SUBMAPS || !coeffs || n < 0 || (n > 0 && (!q || !out)))
    return arg_error("cmm_compose: bad argument");
  for (int k = 0; k < S; ++k)
    if (!coeffs[k]) return arg_error("cmm_compose: null coefficient pointer");
  return launch_compose(mesh->view, coeffs, S, q, n, out, tri, tri_all, jac,
                        (cudaStream_t)stream);
}

int cmm_flow_velocity(const cmm_mesh* mesh, int flow, double T, double alpha, double t, const double* x,
                      int64_t n, double* out, void* stream) {
  if (!mesh || n < 0 || (n > 0 && (!x || !out))) return arg_error("cmm_flow_velocity: bad argument");
  return flow_velocity(mesh->view, flow, T, alpha, t, x, n, out, (cudaStream_t)stream);
}

int cmm_flow_integrate(const cmm_mesh* mesh, int flow, double T, double alpha, int scheme, double t,
                       double dt, const double* x, int64_t n, double* out, void* stream) {
  if (!mesh || n < 0 || (n > 0 && (!x || !out))) return arg_error("cmm_flow_integrate: bad argument");
  return flow_integrate(mesh->view, flow, T, alpha, scheme, t, dt, x, n, out, (cudaStream_t)stream);
}

int cmm_flow_advect_project(const cmm_mesh* mesh, int flow, double T, double alpha, int scheme, double t,
                            double dt, const double* s_pts, const double* tan, const double* prev_coeffs,
                            double eps, double* jets, double* work, void* stream) {
  if (!mesh || mesh->view.kind != kIcosahedral) return arg_error("cmm_flow_advect_project: map mesh expected");
  if (!s_pts || !tan || !jets || !work) return arg_error("cmm_flow_advect_project: null pointer");
  cudaStream_t s = (cudaStream_t)stream;
  int rc = flow_advect_points(mesh->view, flow, T, alpha, scheme, t, dt, s_pts, work, s);
  if (rc) return rc;
  const int64_t nv = mesh->view.nv;
  return launch_project_jets(mesh->view, prev_coeffs, work, work + 3 * nv, tan, eps, jets, s);
}

int cmm_tracer_eval(const cmm_mesh* mesh, int tracer, double t, const double* X, int64_t n, double* out,
                    void* stream) {
  if (!mesh || n < 0 || (n > 0 && (!X || !out))) return arg_error("cmm_tracer_eval: bad argument");
  return launch_tracer(mesh->view, tracer, t, X, n, out, (cudaStream_t)stream);
}

int64_t cmm_query_order_workspace(int64_t n) { return n < 0 ? -1 : order_workspace(n); }

int cmm_query_order(const cmm_mesh* mesh, const double* q, int64_t n, int32_t* perm,
                    int32_t* work, void* stream) {
  if (!mesh || n < 0 || n > INT32_MAX || (n > 0 && (!q || !perm || !work)))
    return arg_error("cmm_query_order: bad argument");
  return launch_query_order(mesh->view, q, n, perm, work, (cudaStream_t)stream);
}

int cmm_assemble_forms(const cmm_mesh* mesh, const double* coeffs, double* forms, void* stream) {
  if (!mesh || mesh->view.kind != kIcosahedral || !coeffs || !forms)
    return arg_error("cmm_assemble_forms: bad argument");
  return launch_assemble_forms(mesh->view, coeffs, forms, (cudaStream_t)stream);
}

int cmm_forms_ff(const cmm_mesh* mesh, const double* forms, float* forms_ff, void* stream) {
  if (!mesh || mesh->view.kind != kIcosahedral || !forms || !forms_ff)
    return arg_error("cmm_forms_ff: bad argument");
  return launch_forms_ff(mesh->view, forms, forms_ff, (cudaStream_t)stream);
}

int cmm_compose_forms(const cmm_mesh* mesh, const double* const* coeffs, const double* const* forms,
                      const float* const* forms_ff, int S, const double* q, int64_t n, const int32_t* perm,
                      double* out, int32_t* tri, int32_t* tri_all, double* jac, void* stream) {
  if (!mesh || mesh->view.kind != kIcosahedral || S < 1 || S > CMM_MAX_SUBMAPS || !coeffs || n < 0 ||
      n > INT32_MAX || (n > 0 && (!q || !out)))
    return arg_error("cmm_compose_forms: bad argument");
  for (int k = 0; k < S; ++k)
    if (!coeffs[k]) return arg_error("cmm_compose_forms: null coefficient pointer");
  return launch_compose(mesh->view, coeffs, S, q, n, out, tri, tri_all, jac, (cudaStream_t)stream, perm,
                        forms, forms_ff);
}

int cmm_compose_ordered(const cmm_mesh* mesh, const double* const* coeffs, int S, const double* q,
                        int64_t n, const int32_t* perm, double* out, int32_t* tri,
                        int32_t* tri_all, double* jac, void* stream) {
  if (!mesh || S < 1 || S > CMM_MAX_SUBMAPS || !coeffs || n < 0 || n > INT32_MAX ||
      (n > 0 && (!q || !out || !perm)))
    return arg_error("cmm_compose_ordered: bad argument");
  for (int k = 0; k < S; ++k)
    if (!coeffs[k]) return arg_error("cmm_compose_ordered: null coefficient pointer");
  return launch_compose(mesh->view, coeffs, S, q, n, out, tri, tri_all, jac,
                        (cudaStream_t)stream, perm);
}

int cmm_stencil_eval(const cmm_mesh* mesh, const double* coeffs, const double* yn,
                     const double* st, int64_t nv, double* out, void* stream) {
  if (!mesh || !coeffs || !yn || !st || !out || nv < 0)
    return arg_error("cmm_stencil_eval: bad argument");
  return launch_stencil_eval(mesh->view, coeffs, yn, st, nv, out, (cudaStream_t)stream);
}

}  // extern "C"
