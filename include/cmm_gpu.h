/*
 * cmm_gpu.h -- C ABI of libcmmgpu.so, the GB300 (sm_103a) implementation of
 * the Characteristic Mapping Method hot path on the sphere.
 *
 * Conventions
 *  - All array arguments of compute calls are DEVICE pointers (for example
 *    torch.Tensor.data_ptr()), FP64 unless stated, C-contiguous.
 *  - `stream` is a cudaStream_t passed as void*; NULL means the legacy
 *    default stream.  Every compute call is asynchronous on that stream.
 *  - Every entry point returns a cmm_status.  Argument errors are detected on
 *    the host and returned at once.  Conditions found by a kernel (a
 *    non-finite value, a query outside every triangle) are OR-ed into the
 *    context's device status word; cmm_mesh_status() reads and clears it.
 *  - cmm_last_error() returns a message for the last failing call on the
 *    calling thread.
 *  - Jet arrays use the reference's layout (C,4,Nv): jets[c][0][v] is
 *    component c of the value at vertex v and jets[j][1+k][v] is the
 *    derivative along axis j of component k.
 *  - Coefficient arrays are owned by the caller and hold, per triangle, a
 *    record of cmm_coeff_stride(C) doubles: ordinate o (0..18) of component c
 *    at offset 3*o + c (C = 3) or o (C = 1).
 *
 * Reference interfaces each entry point replaces are cited as
 * path:line inside the seth-tl/CMM-S2 repository.
 */
#ifndef CMM_GPU_H
#define CMM_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  CMM_OK = 0,
  CMM_ERR_ARG = 1,          /* invalid argument */
  CMM_ERR_MESH = 2,         /* mesh tables inconsistent / not supported */
  CMM_ERR_CUDA = 3,         /* CUDA runtime error */
  CMM_ERR_NONFINITE = 4,    /* status bit: a non-finite value was met */
  CMM_ERR_LOCATE = 5,       /* status bit: a query fell outside its triangle */
  CMM_ERR_TIMEOUT = 6,      /* a bounded wait ran out */
  CMM_ERR_UNSUPPORTED = 7,
  CMM_ERR_NOMEM = 8         /* a host allocation failed */
} cmm_status;

/* Bits of the device status word. */
#define CMM_FLAG_NONFINITE 1
#define CMM_FLAG_LOCATE 2
#define CMM_FLAG_TIMEOUT 4   /* a bounded wait inside a kernel ran out */
#define CMM_FLAG_INDEX 8     /* an index argument (a permutation entry) was out of range; skipped */
/* After a timeout a tensor-core kernel waits (bounded) for its own copies
 * and products still in flight before it releases its tensor memory and
 * returns.  If that drain also runs out, operations of the kernel may still
 * be in flight: this bit is set beside CMM_FLAG_TIMEOUT and the CUDA
 * context must be treated as unusable (reset it before further work). */
#define CMM_FLAG_DRAIN_TIMEOUT 16

const char* cmm_last_error(void);
int cmm_version(void);
/* Number of kernels this library has launched so far in the process
 * (library-call kernels such as cuFFT's not included). */
long long cmm_launch_count(void);

/* ------------------------------------------------------------------ mesh */
typedef struct cmm_mesh cmm_mesh;

/* Build the device tables of an icosahedral refinement of level `level`
 * from the caller's HOST arrays verts (nv,3) and tris (nt,3) (counter-
 * clockwise rows, the reference's triangle order).  Replaces the set-up of
 * spherical_triangulation (cmm_s2/core/mesh_functions.py:29-66, ps_split
 * :92-126): point location runs as a descent through the refinement
 * hierarchy, and the leaf found is reported as the row index of `tris`. */
int cmm_mesh_create(const double* verts, int nv, const int32_t* tris, int nt, int level,
                    cmm_mesh** out);
int cmm_mesh_destroy(cmm_mesh* mesh);
/* Host-only validation of the same inputs (no device work): builds the
 * hierarchy and, if leaf_row is not NULL, writes the row of `tris` of each
 * hierarchy leaf (nt,) in descent order (leaf 4*f+c is child c of node f,
 * children of (a,b,c) ordered (a,mab,mca), (mab,b,mbc), (mca,mbc,c),
 * (mbc,mca,mab)). */
int cmm_mesh_check(const double* verts, int nv, const int32_t* tris, int nt, int level,
                   int32_t* leaf_row);
/* Read (and with clear != 0, reset) the device status word; synchronises
 * `stream`. */
int cmm_mesh_status(cmm_mesh* mesh, void* stream, int* flags, int clear);

/* Number of doubles per triangle record of a coefficient array. */
int cmm_coeff_stride(int ncomp);

/* Point location: containing triangle (row of tris) and un-normalised
 * spherical barycentrics.  q (n,3); tri (n,) int32; bcc (n,3), may be NULL.
 * Replaces spherical_triangulation.query (cmm_s2/core/mesh_functions.py:68-88). */
int cmm_locate(const cmm_mesh* mesh, const double* q, int64_t n, int32_t* tri, double* bcc,
               void* stream);

/* Powell-Sabin ordinates from jets (ncomp,4,nv) -> coeffs (nt, stride).
 * Replaces sphere_diffeomorphism.assemble_coefficients
 * (cmm_s2/core/spherical_spline.py:300-337), spherical_spline
 * .assemble_coefficients (:115-152) and composite_sphere_diffeomorphism
 * .assemble_coefficients (:471-508). */
int cmm_assemble(const cmm_mesh* mesh, const double* jets, int ncomp, double* coeffs,
                 void* stream);

/* Composition X = S_0 o S_1 o ... o S_{S-1}(q): submap S-1 is applied first
 * (cmm_s2/core/spherical_spline.py:365-398); S = 1 is a single map
 * (sphere_diffeomorphism.__call__, :178-205).  coeffs: HOST array of S
 * device pointers to coefficient arrays (ncomp = 3).  q (n,3); out (n,3)
 * unit points.  tri (n,) int32 = triangle of q itself, may be NULL.
 * tri_all (S,n) int32 = triangle used by submap s, may be NULL.
 * jac (n,9) row-major 3x3 tangent Jacobian dX/dq (restated from
 * spherical_spline.gradient :73-111, grad_HBB :700-713 and the
 * normalisation derivative :247-263; eval_grad :208-265 is broken in the
 * reference), may be NULL.  S <= CMM_MAX_SUBMAPS. */
#define CMM_MAX_SUBMAPS 1024
int cmm_compose(const cmm_mesh* mesh, const double* const* coeffs, int S, const double* q,
                int64_t n, double* out, int32_t* tri, int32_t* tri_all, double* jac,
                void* stream);

/* ------------------------------------------------- linear transport */
/* The analytic test flows of cmm_s2/core/dynamical_fields.py, in closed
 * form inside the backward integrators, for linear advection of a tracer
 * (cmm_s2/tests/test_spherical_transport.py).  T: period (the module's
 * T = 1), alpha: tilt of the solid-body rotation (the module's alpha = 0).
 * mesh: the map mesh (its status word receives CMM_FLAG_NONFINITE). */
#define CMM_FLOW_SOLID_BODY 0      /* u_sbr, :18-22 */
#define CMM_FLOW_DEFORM 1          /* u_deform, :24-30 */
#define CMM_FLOW_DEFORM_ROT 2      /* u_deform_rot, :32-42 */
#define CMM_FLOW_STATIC_VORTEX 3   /* u_static_vortex, :57-65 */
#define CMM_FLOW_ROTATING_VORTEX 4 /* u_rotating_vortex, :67-76 */
#define CMM_FLOW_EQUATOR_VORTEX 5  /* equator_vortex, :78-83 */
#define CMM_FLOW_DIVERGENT 6       /* u_div, :97-107 */

/* Velocity V(t, x) of a flow at x (3,n) -> out (3,n). */
int cmm_flow_velocity(const cmm_mesh* mesh, int flow, double T, double alpha, double t, const double* x,
                      int64_t n, double* out, void* stream);

/* cmm_integrate with an analytic flow (any scheme, CMM_RK2 included). */
int cmm_flow_integrate(const cmm_mesh* mesh, int flow, double T, double alpha, int scheme, double t,
                       double dt, const double* x, int64_t n, double* out, void* stream);

/* cmm_advect_project with an analytic flow: advect_project_sphere(interp,
 * integrator, t, dt, U, identity) of evolution_functions.py:136-142 with
 * U one of the flows above.  work: 15*nv doubles. */
int cmm_flow_advect_project(const cmm_mesh* mesh, int flow, double T, double alpha, int scheme, double t,
                            double dt, const double* s_pts, const double* tan, const double* prev_coeffs,
                            double eps, double* jets, double* work, void* stream);

/* Tracer fields at points X (n,3) -> out (n,): the initial conditions of
 * dynamical_fields.py and the smooth test function of
 * tests/test_spherical_transport.py:36-38.  t: time argument of the vortex
 * fields (ignored by the others). */
#define CMM_TRACER_COSINE_BELL 0        /* cosine_bell, :122-137 */
#define CMM_TRACER_SLOTTED_CYLINDERS 1  /* IC_SC, :139-157 */
#define CMM_TRACER_STATIC_VORTEX 2      /* static_vort_IC, :85-88 */
#define CMM_TRACER_ROTATING_VORTEX 3    /* rotating_vort_IC, :90-95 */
#define CMM_TRACER_SMOOTH_TEST 4        /* test_func of the transport test */
#define CMM_TRACER_RANDOM_SH 5          /* random_initial_condition, :158-172: the
                                           degree-32 series of numpy's seed-42 draws;
                                           first call outside a stream capture */
int cmm_tracer_eval(const cmm_mesh* mesh, int tracer, double t, const double* X, int64_t n, double* out,
                    void* stream);

/* Query order for cmm_compose_ordered: perm (n,) int32 receives the query
 * ids grouped by the level-4 hierarchy cell holding each query (a counting
 * sort; the order inside a cell is unspecified), so that neighbouring threads of the
 * composition gather neighbouring coefficient records and share them in
 * L1/L2 instead of re-reading DRAM.  work: cmm_query_order_workspace(n)
 * int32 device scratch.  n <= INT32_MAX.  No counterpart in the reference
 * (its queries are processed in caller order by numpy). */
int64_t cmm_query_order_workspace(int64_t n);
int cmm_query_order(const cmm_mesh* mesh, const double* q, int64_t n, int32_t* perm,
                    int32_t* work, void* stream);

/* cmm_compose with the queries processed in the order perm (a permutation
 * of 0..n-1, e.g. from cmm_query_order); every output stays in its query's
 * own slot and is bitwise equal to cmm_compose's.  An entry outside
 * [0, n) is skipped and sets CMM_FLAG_INDEX. */
int cmm_compose_ordered(const cmm_mesh* mesh, const double* const* coeffs, int S, const double* q,
                        int64_t n, const int32_t* perm, double* out, int32_t* tri,
                        int32_t* tri_all, double* jac, void* stream);

/* Map forms: the same Powell-Sabin patches as a coefficient record,
 * re-expressed per sub-triangle and component as the homogeneous quadratic
 * form P(p) = p^T Q p in the ambient point (the sub-triangle barycentrics
 * are linear in p, so each patch is exactly such a form; stored as Qxx,
 * Qyy, Qzz, 2Qxy, 2Qxz, 2Qyz).  Q is assembled in double-double from the
 * record's ordinates and the location record's inverse vertex rows, then
 * rounded once; evaluating p^T Q p costs 24 FP64 operations against ~40
 * for barycentrics plus the Bernstein sum, and with the Powell-Sabin
 * sub-triangle chosen from FP32 barycentrics (FP64 when a pair is within
 * the FP32 error bound) the composition needs no FP64 location at all.
 * Same values to rounding (measured ~1e-16 per evaluation; the Bernstein
 * sum carries ~1e-14 from the barycentric product).  No counterpart in the
 * reference.  forms: (Nt, CMM_FORM_STRIDE) doubles. */
#define CMM_FORM_STRIDE 112
int cmm_assemble_forms(const cmm_mesh* mesh, const double* coeffs, double* forms, void* stream);
/* Low floats of the float-float split of form records, for the Jacobian
 * pushes (which run in float-float): per sub-triangle and component the
 * entries Qxx, Qyy, Qzz, Qxy, Qxz, Qyz of the symmetric matrix, each split
 * as hi = the double truncated to 24 significand bits, lo = the next 24
 * bits truncated (the cross terms halved, exact); lo is stored, hi is
 * re-derived from the double.  The composition then skips most of the
 * split's integer work; the results are bitwise the same.  Pays with the
 * queries grouped by coarse cell (cmm_query_order); in random order the
 * 72 more bytes gathered per evaluation cost more than they save.
 * forms_ff: (Nt, CMM_FORM_FF_STRIDE) floats. */
#define CMM_FORM_FF_STRIDE 112
int cmm_forms_ff(const cmm_mesh* mesh, const double* forms, float* forms_ff, void* stream);
/* cmm_compose / cmm_compose_ordered with map forms: forms is a HOST array
 * of S device pointers to form records (an entry may be NULL: that submap
 * is evaluated from its coefficient record) or NULL; forms_ff a HOST array
 * of S device pointers to their low floats (cmm_forms_ff; used when every
 * submap with a form record has them) or NULL; perm may be NULL (caller
 * order).  Outputs as cmm_compose's. */
int cmm_compose_forms(const cmm_mesh* mesh, const double* const* coeffs, const double* const* forms,
                      const float* const* forms_ff, int S, const double* q, int64_t n, const int32_t* perm,
                      double* out, int32_t* tri, int32_t* tri_all, double* jac, void* stream);

/* Stencil evaluation: locate each vertex foot point yn[:,v] (3,nv), then
 * evaluate the 4 stencil foot points st (3,4,nv) in that same Powell-Sabin
 * sub-triangle, un-normalised -> out (3,4,nv).  Replaces
 * sphere_diffeomorphism.stencil_eval (cmm_s2/core/spherical_spline.py:268-298). */
int cmm_stencil_eval(const cmm_mesh* mesh, const double* coeffs, const double* yn,
                     const double* st, int64_t nv, double* out, void* stream);

/* ------------------------------------------------------ velocity mesh */
/* MWSS lat-lon velocity mesh at band-limit L from the caller's HOST arrays:
 * ring colatitudes theta (L+1), longitudes phi (2L), ring points grid
 * (3, (L+1)*2L) and mesh vertices verts (2+(L-1)*2L, 3) (north pole, the
 * interior rings row by row, south pole).  Replaces
 * structure_spherical_triangulation (cmm_s2/core/mesh_functions.py:175-194,
 * grid_assemble/full_assembly :352-412).  The handle works with
 * cmm_locate (structured O(1) query, :196-282) and cmm_assemble. */
int cmm_velmesh_create(int L, const double* theta, const double* phi, const double* grid,
                       const double* verts, cmm_mesh** out);

/* Velocity at points x (3,n) at time t from nvs (1..3) time levels of
 * coefficients (HOST array of nvs device pointers) sampled at ts0,
 * ts0+dt, ts0+2dt -> out (3,n).  Replaces spline_interp_velocity.__call__
 * (cmm_s2/core/spherical_spline.py:570-615). */
int cmm_velocity_eval(const cmm_mesh* velmesh, const double* const* vel_coeffs, int nvs,
                      double ts0, double t, double dt, const double* x, int64_t n, double* out,
                      void* stream);

/* Backward foot points of x (3,n) over one step from t+dt to t, projected
 * onto the sphere after each stage -> out (3,n).  scheme 0: Euler_step_proj,
 * 1: improved_Euler_proj, 2: RK4_proj, 3: RK2_proj
 * (cmm_s2/core/evolution_functions.py:19-80; RK3_proj :35-47 passes three
 * arguments to the one-argument div_norm and cannot run, so it has no
 * counterpart).  The adjoint entry points take schemes 0-2. */
#define CMM_EULER 0
#define CMM_IMPROVED_EULER 1
#define CMM_RK4 2
#define CMM_RK2 3
int cmm_integrate(const cmm_mesh* velmesh, const double* const* vel_coeffs, int nvs, double ts0,
                  int scheme, double t, double dt, const double* x, int64_t n, double* out,
                  void* stream);

/* Scratch doubles cmm_advect_project needs for a mesh of nv vertices. */
int64_t cmm_advect_workspace(const cmm_mesh* mesh);

/* One CMM map update (advect_project_sphere,
 * cmm_s2/core/evolution_functions.py:117-142): integrate the mesh vertices
 * and the stencil points s_pts (3,4,nv) backward through the velocity,
 * evaluate the previous map (coefficients prev_coeffs; NULL = identity) at
 * the stencil foot points in the sub-triangle of each vertex foot point,
 * and write the new jets (3,4,nv) from the stencil average and centred
 * differences in the tangent frames tan (2,nv,3) with step eps
 * (spline_proj_sphere, :90-113).  work: cmm_advect_workspace(mesh) doubles;
 * on return it holds the vertex foot points (3,nv) followed by the stencil
 * foot points (3,4,nv). */
int cmm_advect_project(const cmm_mesh* mesh, const cmm_mesh* velmesh,
                       const double* const* vel_coeffs, int nvs, double ts0, int scheme, double t,
                       double dt, const double* s_pts, const double* tan,
                       const double* prev_coeffs, double eps, double* jets, double* work,
                       void* stream);

/* The same map update as cmm_advect_project, for callers that cannot
 * allocate device memory -- for instance an application that has handed
 * all of the GPU's memory to its own pool, or a solver loop that must not
 * call cudaMalloc/cudaFree, which can synchronise the whole device.  It
 * allocates nothing: its foot-point scratch (15 doubles per vertex) is a
 * fixed array compiled into the library, present on every GPU that loads
 * it until the process exits.  No counterpart in the reference.
 *  - Meshes of at most 10242 vertices (icosahedral level 5); larger ones
 *    are rejected with CMM_ERR_ARG (use cmm_advect_project with a
 *    workspace).
 *  - The first call on each device looks up that device's copy of the
 *    scratch array (cudaGetSymbolAddress) with the device current; make
 *    that first call before any stream capture.  The address is kept for
 *    the life of the process: after cudaDeviceReset (or anything else
 *    that destroys the device's primary context) the library's module is
 *    loaded again and the kept address is stale, so do not call this entry
 *    point on a device that has been reset.
 *  - All calls on a device share the one array and it keeps the last
 *    call's contents (every entry is rewritten before it is read, so
 *    nothing needs clearing): calls that overlap on the GPU, on different
 *    streams or from different threads, race and must be serialised by
 *    the caller. */
int cmm_advect_project_noalloc(const cmm_mesh* mesh, const cmm_mesh* velmesh,
                               const double* const* vel_coeffs, int nvs, double ts0, int scheme,
                               double t, double dt, const double* s_pts, const double* tan,
                               const double* prev_coeffs, double eps, double* jets, void* stream);

/* ------------------------------------------------------------ vorticity */
/* Initial vorticity fields: the barotropic fields of
 * cmm_s2/core/dynamical_fields.py:181-214 and benchmark fields. */
#define CMM_VORT_NONE 0
#define CMM_VORT_ROSSBY_HAURWITZ 1 /* params[0] = t  (rossby_wave, :205-210) */
#define CMM_VORT_ZONAL_JET 2       /* zonal_jet, :181-186 */
#define CMM_VORT_PERTURBED_JET 3   /* perturbed_zonal_jet, :188-192 */
#define CMM_VORT_MULTI_JET 4       /* multi_jet, :195-198 */
#define CMM_VORT_GAUSSIAN_VORTEX 5 /* gaussian_vortex, :200-203 */
#define CMM_VORT_GAUSSIAN_JETS 6   /* params: amplitude, width (rad), n <= 9,
                                      latitudes (rad): sum A exp(-((lat-l_j)/w)^2) */
#define CMM_VORT_PERTURBED_RH 7    /* perturbed_rossby_wave, :213-215 */

/* omega at the sample rings of `velmesh` (L+1,2L) from the back-traced
 * sample points X ((L+1)*2L, 3): omega0(X) + 2 rot cos(theta(X)) -
 * 2 rot cos(theta_ring) (cmm_s2/core/spherical_simulations.py:269-272),
 * omega0 = field `kind` plus, when sh is not NULL, the real orthonormal
 * spherical-harmonic series sh (lmax+1, 2lmax+1) (column l+m; m>0 cos,
 * m<0 sin, both with sqrt2; lmax <= 128), plus, when spline is not NULL, the scalar
 * Powell-Sabin spline with ncomp=1 coefficients `spline` on `velmesh`
 * (the spherical_spline a caller builds with cmm_sht_scalar_jets +
 * cmm_assemble, as project_onto_S12 does,
 * cmm_s2/core/spherical_harmonic_tools.py:108-142). */
int cmm_vorticity_eval(const cmm_mesh* velmesh, int kind, const double* params, int nparams,
                       const double* sh, int lmax, const double* spline, double rot_rate,
                       const double* X, double* omega, void* stream);

/* ------------------------------------------- spherical-harmonic transforms */
/* MWSS transforms at band-limit L (samples on L+1 rings x 2L longitudes,
 * real fields).  Coefficients use an m-major half layout: alm[m][l]
 * complex (interleaved re,im doubles), 0 <= m <= l < L, entries with l < m
 * zero; negative orders follow from a_{l,-m} = (-1)^m conj(a_lm).
 * The plan owns its FFT plans and scratch buffers. */
typedef struct cmm_sht cmm_sht;
typedef struct cmm_sht_batch cmm_sht_batch;
int cmm_sht_create(int L, cmm_sht** out);
int cmm_sht_destroy(cmm_sht* plan);

/* Arithmetic of the 12-field Legendre synthesis of cmm_sht_velocity /
 * cmm_sht_inverse: CMM_SHT_FP64 (default; FP64 recurrence and sums) or
 * CMM_SHT_SPLIT_BF16: each factor split into bf16 hi + lo, products
 * hi*hi + hi*lo + lo*hi on the tensor cores (tcgen05) accumulated in FP32
 * per 64-term chunk and in compensated (Kahan) FP32 sums across chunks,
 * for both the forward
 * analysis (cmm_sht_forward, the analysis inside cmm_sht_velocity) and the
 * 12-field synthesis, whose ring FFTs then run in FP32; Pbar tables
 * (about 4.4 GB at L = 1024) are built when the mode is first selected.
 * Measured error about 4e-6 (analysis) and 6e-6 (synthesis) of the largest
 * coefficient / sample.  The pyssht calls this replaces work in FP64. */
#define CMM_SHT_FP64 0
#define CMM_SHT_SPLIT_BF16 1
int cmm_sht_set_precision(cmm_sht* plan, int mode);
/* Schedule of the split-BF16 synthesis kernel: 1 (default) warp-specialised
 * -- a copy warp, an MMA warp and four drain warps run concurrently; 0 --
 * the same warps take each role in turn.  Both accumulate each 64-degree
 * chunk in FP32 in tensor memory and add the chunk partials into
 * compensated FP32 register sums in the same order: bitwise the same
 * results.  No counterpart in the reference. */
int cmm_sht_set_schedule(cmm_sht* plan, int schedule);
/* Share the Legendre tables of `src` (another plan of the same L) instead
 * of building them again; plans of one band-limit then share one copy and
 * still run concurrently (each keeps its own data tiles and FFT scratch).
 * src in CMM_SHT_SPLIT_BF16 mode: `plan` is put in that mode on src's
 * split-bf16 Pbar tables (~4.4 GB at L = 1024).  src in CMM_SHT_FP64 mode:
 * `plan` keeps its precision and takes src's FP64 Pbar tables (built on
 * src first; 0.8 GB at L = 512) and table mode; CMM_ERR_ARG when src's
 * FP64 stages run without tables (cmm_sht_set_tables).  Synchronises. */
int cmm_sht_share_tables(cmm_sht* plan, cmm_sht* src);
/* Failure-path self-test: runs the tensor-core kernels' bounded mbarrier
 * wait on a barrier that nothing ever completes, with a limit of `polls`
 * (1..2^20) polls; the wait runs out, the block sets CMM_FLAG_TIMEOUT in the
 * plan's status word (read with cmm_sht_status) and returns, leaving the
 * context usable.  No counterpart in the reference. */
int cmm_sht_timeout_selftest(cmm_sht* plan, long long polls, void* stream);
/* FP64 Legendre stages from tabulated Pbar_lm (analysis and synthesis as
 * table contractions; 0.8 GB at L = 512, 6.5 GB at L = 1024) instead of
 * the on-the-fly recurrence: mode 0 (default) for L <= 512, 1 for any
 * L <= 1024, -1 never.  The tables are built at the next FP64 stage that
 * runs outside a stream capture, which then synchronises its stream once,
 * so later calls of the plan on any stream find them complete.  No
 * counterpart in the reference. */
int cmm_sht_set_tables(cmm_sht* plan, int mode);
/* Release the FP64 inverse scratch (about 400 MB at L = 1024) and, at
 * the FP64 Pbar tables (cmm_sht_set_tables); each is allocated
 * again at its next use (the tables only by a call outside a stream
 * capture; inside one the FP64 stages use their recurrence kernels).
 * Synchronises the device. */
int cmm_sht_trim(cmm_sht* plan);
/* Read (and with clear != 0, reset) the plan's device status word
 * (CMM_FLAG_TIMEOUT); synchronises `stream`. */
int cmm_sht_status(cmm_sht* plan, void* stream, int* flags, int clear);
/* A batch of 1 to CMM_SHT_BATCH_MAX split-BF16 plans of one band-limit
 * (distinct, in no other batch; best with shared tables,
 * cmm_sht_share_tables) whose forward Legendre analyses run as one
 * tensor-core launch: member b's field occupies columns 2b, 2b+1 of the
 * N = 16 data tiles, so every Pbar tile streamed from HBM feeds all
 * members.  Used by the split device-driven step (cmm_bve_step_pre /
 * cmm_sht_batch_analysis / cmm_bve_step_post) of ensemble members of one
 * band-limit; each member's coefficients are bitwise those of its own
 * analysis.  Destroy the batch before its plans (a plan destroyed first
 * makes the batch's analysis return CMM_ERR_ARG).  Create and destroy
 * synchronise the device.  No counterpart in the reference. */
#define CMM_SHT_BATCH_MAX 8
int cmm_sht_batch_create(cmm_sht* const* plans, int n, cmm_sht_batch** out);
int cmm_sht_batch_destroy(cmm_sht_batch* batch);
/* The batch's analysis: after every member's cmm_bve_step_pre on this or
 * an earlier-joined stream; timeouts are reported in the first member
 * plan's status word. */
int cmm_sht_batch_analysis(cmm_sht_batch* batch, void* stream);
/* Forward transforms (as cmm_sht_forward) of one field per member through
 * the batched analysis: samples[b] (L+1,2L) -> alm[b] (L,L) complex, HOST
 * arrays of the batch's member count of device pointers. */
int cmm_sht_batch_forward(cmm_sht_batch* batch, const double* const* samples, double* const* alm,
                          void* stream);

/* samples (L+1,2L) -> alm (L,L) complex.  Replaces pyssht.forward(...,
 * Method="MWSS", Reality=True) as called by inv_Laplacian
 * (cmm_s2/core/spherical_harmonic_tools.py:16). */
int cmm_sht_forward(cmm_sht* plan, const double* samples, double* alm, void* stream);

/* nf (1 or 12) coefficient fields (nf,L,L) complex -> samples
 * (nf,L+1,2L).  Replaces pyssht.inverse(..., Method="MWSS", Reality=True)
 * (cmm_s2/core/spherical_harmonic_tools.py:84,91). */
int cmm_sht_inverse(cmm_sht* plan, const double* alm, int nf, double* samples, void* stream);

/* Vorticity samples omega (L+1,2L) on the velocity mesh's rings -> velocity
 * jets (3,4,Nv_u) of the velocity mesh: inv_Laplacian, the angular-momentum
 * operators and the 12 inverse transforms of project_stream with its
 * tangent projection and pole handling
 * (cmm_s2/core/spherical_harmonic_tools.py:14-19, 49-105).  psi (L,L)
 * complex receives the stream function coefficients when not NULL; with
 * omega NULL, psi is the input instead (project_stream alone). */
int cmm_sht_velocity(cmm_sht* plan, const cmm_mesh* velmesh, const double* omega, double* psi,
                     double* vel_jets, void* stream);

/* Scalar jets (4, Nv_u) on the velocity mesh's vertices of the real field
 * with coefficients alm (L,L) complex: value, then the tangent gradient
 * from the angular-momentum operators (project_onto_S12,
 * cmm_s2/core/spherical_harmonic_tools.py:108-142).  With cmm_assemble
 * (ncomp = 1) this builds the scalar spherical_spline of the field. */
int cmm_sht_scalar_jets(cmm_sht* plan, const cmm_mesh* velmesh, const double* alm, double* jets,
                        void* stream);

/* Storage of this velocity mesh's velocity coefficient records (ncomp = 3):
 * CMM_REC_FP64 (default; (nt, 64) doubles) or CMM_REC_FP32 ((nt, 64)
 * floats: cmm_assemble with ncomp = 3 writes FP32 ordinates computed in
 * FP32 from the FP64 jets, and velocity evaluation forms the patches and
 * their time combination in FP32; location, barycentrics, the RK4
 * accumulation and the sphere projection stay FP64).  For the mixed form,
 * whose velocities carry the split-BF16 transform's ~1e-5 relative error;
 * halves the records' memory and traffic.  Scalar (ncomp = 1) records stay
 * FP64.  Not a reference function: its velocity records are FP64. */
#define CMM_REC_FP64 0
#define CMM_REC_FP32 1
/* CMM_REC_FP32 plus the analytic initial-vorticity fields of
 * cmm_vorticity_eval (not the SH series or the spline term) evaluated in
 * FP32 from FP32 angles (relative error ~1e-7), cos(theta) as z/|X|. */
#define CMM_REC_MIXED 2
int cmm_velmesh_set_records(cmm_mesh* velmesh, int precision);

/* Threads per block of a tunable kernel launched on this mesh (set by an
 * autotuner from measured timings; 0 restores the default): composition
 * and location on a map mesh, the map update's foot-point kernel on a map
 * mesh, the vorticity kernel on a velocity mesh.  threads: 0 or a multiple
 * of 32 in [32, 256].  Launch shape only: results do not depend on it. */
#define CMM_TUNE_COMPOSE 0
#define CMM_TUNE_ADVECT 1
#define CMM_TUNE_VORTICITY 2
#define CMM_TUNE_LOCATE 3
int cmm_mesh_set_block(cmm_mesh* mesh, int kernel, int threads);

/* Compiled variant of a tunable kernel launched on this mesh (set by an
 * autotuner from measured timings; 0 restores the default).  The
 * composition kernels are compiled for several register budgets, named by
 * the resident 256-thread blocks per SM they allow: with Jacobians 2, 3 or
 * 4 (128, 80 or 64 registers a thread; default 4), points only 4 or 6 (64
 * or 40; default 4).  Fewer registers hide more gather latency, more avoid
 * spills.  Results do not depend on the variant.  No counterpart in the
 * reference. */
#define CMM_VARIANT_COMPOSE_JAC 0
#define CMM_VARIANT_COMPOSE 1
int cmm_mesh_set_variant(cmm_mesh* mesh, int knob, int value);

/* ---------------------------------------------- device-driven BVE steps */
/* The main-loop body of euler_simulation_sphere_remapping
 * (cmm_s2/core/spherical_simulations.py:263-294) as one enqueue per step:
 * map update (RK4, cmm_advect_project), its assembly, the sample points
 * through the submap stack and the current map (cmm_compose), the
 * vorticity there (cmm_vorticity_eval), the velocity jets
 * (cmm_sht_velocity) assembled into the oldest velocity slot, then the
 * driver's bookkeeping (remap into the stack every n_maps steps and at
 * step Nt, velocity-slot rotation, ts0, the next step's RK4 stage weights)
 * done on the device.  The kernels read everything that varies between
 * steps from a device-resident state, so the launches of every step are
 * identical and a CUDA graph captured from one cmm_bve_step replays all
 * later steps (several runs' graphs can be captured into one).  Results
 * are bit-identical to the same run driven step by step from the host.
 * No counterpart function in the reference (its loop is Python).
 * All pointers are device buffers owned by the caller, except `stack` and
 * `stack_jets`: host arrays of n_stack device pointers (copied at create;
 * stack_jets may be NULL). */
typedef struct cmm_bve cmm_bve;
typedef struct {
  const cmm_mesh* mesh;       /* icosahedral map mesh */
  const cmm_mesh* velmesh;    /* MWSS velocity mesh of band-limit L */
  cmm_sht* sht;               /* plan of band-limit L (precision as set) */
  int vort_kind, nparams;     /* initial vorticity, as cmm_vorticity_eval */
  double vort_params[12];
  const double* sh;
  int lmax;
  const double* spline;
  double rot_rate;
  double tspan_step;          /* T / Nt: tspan[k] = k * tspan_step, dt */
  int Nt, n_maps;
  double eps;                 /* stencil half-width (1e-5) */
  const double* s_pts;        /* (3,4,Nv) stencil points */
  const double* tan;          /* (2,Nv,3) tangent frames */
  const double* id_jets;      /* (3,4,Nv) identity jets */
  const double* sample_pts;   /* (Q,3) MWSS sample points, Q = (L+1) 2L */
  double* jets;               /* (3,4,Nv) current map jets */
  double* coeffs_cur;         /* (Nt_map, 64) current map coefficients */
  double* work;               /* cmm_advect_workspace(mesh) doubles */
  double* X;                  /* (Q,3) back-traced sample points */
  double* omega;              /* (L+1, 2L) vorticity samples */
  double* vel_jets;           /* (3,4,Nv_u) velocity jets */
  double* vel[3];             /* velocity coefficient slots, oldest first */
  int n_stack;                /* stack slots (>= remaps of the run) */
  double* const* stack;
  double* const* stack_jets;
  /* state after the bootstrap (spherical_simulations.py:216-261) */
  int k;                      /* tspan index of the next step's start */
  int count, nc, identity;
  double ts0;
  /* map-form records of the stack slots (host array of n_stack device
   * pointers to (Nt_map, CMM_FORM_STRIDE) records, copied at create), or
   * NULL: each remap then also assembles the slot's forms and the
   * composition evaluates the stack through them */
  double* const* stack_forms;
} cmm_bve_desc;
/* Set-up call: uploads the state on the legacy default stream and
 * synchronises the device, so it must not be called while a stream of
 * the device is being captured.  A failed host allocation returns
 * CMM_ERR_NOMEM. */
int cmm_bve_create(const cmm_bve_desc* desc, cmm_bve** out);
int cmm_bve_destroy(cmm_bve* bve);
/* Enqueue one step on `stream` (no host synchronisation, capturable). */
int cmm_bve_step(cmm_bve* bve, void* stream);
/* The same step in two halves around a batched analysis, for a run whose
 * SHT plan is in a batch (cmm_sht_batch_create): _pre runs the step up to
 * the forward transform's data tiles (written into the member's batch
 * slot), cmm_sht_batch_analysis then contracts all members' tiles, and
 * _post runs the rest (stream function, velocity jets, assembly, remap,
 * bookkeeping).  Bitwise the same step as cmm_bve_step. */
int cmm_bve_step_pre(cmm_bve* bve, void* stream);
int cmm_bve_step_post(cmm_bve* bve, void* stream);
/* Read the device state (synchronises `stream`). */
int cmm_bve_state(cmm_bve* bve, void* stream, int* count, int* nc, int* identity);

/* ------------------------------------------------------------ adjoints */
/* Reverse-mode twins of the forward calls: each takes the cotangent of its
 * forward call's output and accumulates (+=, unless stated) the cotangents
 * of the inputs -- the exact transpose of the linearisation of the forward
 * call's discrete arithmetic, with the piecewise choices (triangle,
 * Powell-Sabin sub-triangle) held fixed.  Shared records are accumulated
 * with FP64 atomics.  No counterpart in the reference, which has no
 * derivatives; used by the gradient of a final-time vorticity misfit with
 * respect to the initial spherical-harmonic coefficients. */
/* cmm_assemble (ncomp = 3, FP64 records): grad_jets (3,4,Nv) += A^T grad_coeffs. */
int cmm_assemble_bwd(const cmm_mesh* mesh, const double* grad_coeffs, double* grad_jets, void* stream);
/* cmm_compose without Jacobians (S <= 256): grad_coeffs[s] (Nt, 64) and
 * grad_q (n,3, may be NULL) += ; work: 3 S n doubles. */
int cmm_compose_bwd(const cmm_mesh* mesh, const double* const* coeffs, int S, const double* q, int64_t n,
                    const double* grad_out, double* const* grad_coeffs, double* grad_q, double* work,
                    void* stream);
/* cmm_vorticity_eval for kind CMM_VORT_NONE with a series sh (no spline):
 * grad_X (Q,3) += omega_bar (grad omega0 + 2 rot grad cos theta) with
 * grad omega0 = -X x (iL omega0)(X) from dsh, the three real series
 * (3, lmax+1, 2 lmax+1) of iL_x, iL_y, iL_z applied to sh (NULL: the
 * series term is left out); grad_sh (lmax+1, 2 lmax+1) += sum omega_bar Y. */
int cmm_vorticity_bwd(const cmm_mesh* velmesh, const double* dsh, int lmax, double rot_rate,
                      const double* X, const double* grad_omega, double* grad_X, double* grad_sh,
                      void* stream);
/* cmm_advect_project (FP64 velocity records): grad_vel[l] (Nt_u, 64) and
 * grad_prev (Nt, 64; NULL when prev_coeffs is NULL or not wanted) += the
 * transposes applied to grad_jets (3,4,Nv); the stencil and vertex start
 * points are constants.  work: cmm_advect_workspace(mesh) + 12 Nv doubles. */
int cmm_advect_project_bwd(const cmm_mesh* mesh, const cmm_mesh* velmesh, const double* const* vel_coeffs,
                           int nvs, double ts0, int scheme, double t, double dt, const double* s_pts,
                           const double* tan, const double* prev_coeffs, double eps, const double* grad_jets,
                           double* const* grad_vel, double* grad_prev, double* work, void* stream);
/* cmm_sht_velocity (omega -> velocity jets, FP64 plan): grad_omega
 * (L+1, 2L) = transpose applied to grad_jets (3,4,Nv_u) (overwritten). */
int cmm_sht_velocity_bwd(cmm_sht* plan, const cmm_mesh* velmesh, const double* grad_jets, double* grad_omega,
                         void* stream);

/* Angular power of a real field's coefficients alm (L,L) complex:
 * power[l] = sum over m = -l..l of |a_lm|^2 (L doubles).  Enstrophy is
 * sum_l power[l]; energy_spectrum (cmm_s2/core/spherical_harmonic_tools.py:
 * 157-163) is power[0], power[l] / (l (l+1)). */
int cmm_sht_power(cmm_sht* plan, const double* alm, double* power, void* stream);

#ifdef __cplusplus
}
#endif
#endif
