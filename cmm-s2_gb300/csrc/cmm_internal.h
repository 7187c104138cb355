// Internal declarations shared by the host and device translation units of
// libcmmgpu.so.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>

#include "../../include/cmm_gpu.h"

namespace cmm {

// Per-triangle location record (doubles): rows r1,r2,r3 of the inverse of
// the vertex matrix [v1 v2 v3] (bcc_i = r_i . q), then |v1+v2+v3|,
// |v1+v2|, |v2+v3|, |v3+v1|, 3 doubles of padding.
constexpr int kLocStride = 16;
// Per-triangle assembly factors (doubles): for each of the 9 gradient
// ordinates 3..11 (a_x, a_y, a_z, b) with c = a . grad f(v) - b f(v);
// then the edge-midpoint barycentrics E0[0],E0[1],E1[1],E1[2],E2[0],E2[2]
// used by ordinates 12..17, the centre barycentrics mid[0..2] (ordinate
// 18) and 3 doubles of padding.
constexpr int kAsmStride = 48;
// On the device the 45 used factors are stored factor-major,
// tri_asm[j * nt + t], so that a warp's loads of one factor coalesce.
constexpr int kAsmFactors = 45;
constexpr int kWalkStride = 16;     // per-row walk record: 3 x float4 + padding
constexpr int kWalkMax = 64;        // walk steps before falling back to the descent
constexpr int kCoeffStride3 = 64;   // 19 ordinates x 3 components, padded
constexpr int kCoeffStride1 = 24;   // 19 ordinates, padded
// Map-form record (doubles per triangle): for each of the 6 Powell-Sabin
// sub-triangles (kSubIndex) and each component the homogeneous quadratic
// form P(p) = p^T Q p as (Qxx, Qyy, Qzz, 2Qxy, 2Qxz, 2Qyz), 108 used.
constexpr int kFormStride = 112;
// Low floats of a map-form record's float-float split (floats per
// triangle), for the Jacobian pushes: per sub-triangle (18 floats) and
// component (6) the symmetric matrix entries Qxx, Qyy, Qzz, Qxy, Qxz, Qyz
// as the low float of ff_of (the cross terms halved, exact); the high
// float is re-derived from the double's bits (ff_hi).  108 used.
constexpr int kFormFFStride = 112;

// Device view of an icosahedral mesh.
struct MeshView {
  int level, nv, nt;
  const double* verts;      // (nv,4) x,y,z,0
  const int4* tri_v;        // (nt) vertex ids of each reference row
  const double* tri_loc;    // (nt, kLocStride)
  const double* tri_asm;    // (kAsmFactors, nt), factor-major
  const double* root;       // 20 faces x 12: centroid(3), edge normals ab,bc,ca (9)
  const float* root_f;      // same, FP32
  const int* root_adj;      // 20 x 3: face across edge ab, bc, ca
  const double* node_n;     // hierarchy nodes x 9: normals n0,n1,n2 (levels 0..level-1)
  const float* node_nf;     // same, FP32, unit normals
  const int* leaf_row;      // (nt) hierarchical leaf -> reference row
  // walk location (locate_row): per row kWalkStride floats -- for each edge
  // (v0v1, v1v2, v2v0) its inward unit normal (FP32) and the row across it
  // (bit pattern in the 4th float), then the barycentric scales s_0..s_2
  // (b_i = s_i n_(i+1,i+2) . q) -- the FP64 normals (kWalkStride
  // doubles per row, 9 used) and a cube-map jump table of 6 jump_res^2
  // starting rows (NULL until built: the hierarchy descent is used)
  const float* walk_f;
  const double* walk_d;
  const int* jump;
  int jump_res;
  int* status;              // device status word
  // MWSS lat-lon velocity mesh (kind == kLatLon)
  int kind;                 // kIcosahedral or kLatLon
  int L;                    // band-limit: L+1 rings of 2L points
  const double* theta;      // (L+1) ring colatitudes
  const double* phi;        // (2L) longitudes
  const double* grid;       // ((L+1)*2L, 4) ring points x,y,z,0
  // lat-lon side-test normals, 4 doubles per (ring, sector p): ring_n =
  // grid(ring, p) x grid(ring, p+1), diag_n = grid(ring, p) x
  // grid(ring+1, p+1) (rings 0..L-1), each product rounded as numpy's cross
  const double* ring_n;
  const double* diag_n;
  double dphi, dthe;
  // velocity records (ncomp = 3) in FP32 (cmm_velmesh_set_records):
  // (nt, 64) floats, assembled from the FP32 copy of the factors
  int rec32;
  const float* tri_asm_f;   // (kAsmFactors, nt), factor-major, when rec32
  int field32;              // analytic initial vorticity fields in FP32
  const float* tri_loc_f;   // (nt, kLocStride) FP32 copy of the location records, when rec32
  float phi0_f, dphi_f, the0_f, dthe_f;   // FP32 copies of phi[0], dphi, theta[0], dthe
  // recurrence table of the orthonormal associated Legendre functions for
  // real SH series of degree <= kShTableMax: sh_ab[2 (m (kShTableMax+1) + l)]
  // = (a_lm, b_lm), sh_fm[m] = sqrt((2m+1)/(2m))
  const double* sh_ab;
  const double* sh_fm;
  // launch shapes chosen by an autotuner (cmm_mesh_set_block), threads per
  // block of the tunable kernels on this mesh; 0 = the library default
  int block[4];
  // compiled variants chosen by an autotuner (cmm_mesh_set_variant): the
  // register budget of the composition kernels, as resident 256-thread
  // blocks per SM; 0 = the library default
  int variant[2];
};

// Tunable kernels (index into MeshView::block).
constexpr int kTuneCompose = 0, kTuneAdvect = 1, kTuneVorticity = 2, kTuneLocate = 3;
inline int block_of(const MeshView& m, int k, int dflt) { return m.block[k] > 0 ? m.block[k] : dflt; }
// Threads per block for n work items: the tuned size when one is set, else
// the default, or for small n a smaller multiple of 32 so that the grid
// covers each of the 152 SMs twice (a few thousand FP64-heavy points in
// default-size blocks would leave most SMs idle).
constexpr int kNumSMs = 152;
inline int small_block(int64_t n, int dflt) {
  const int64_t want = (n + 2 * kNumSMs - 1) / (2 * kNumSMs);
  const int b = (int)((want + 31) / 32 * 32);
  return b < 32 ? 32 : (b > dflt ? dflt : b);
}
inline int block_for(const MeshView& m, int k, int dflt, int64_t n) {
  return m.block[k] > 0 ? m.block[k] : small_block(n, dflt);
}

constexpr int kShTableMax = 128;
constexpr int kIcosahedral = 0;
constexpr int kLatLon = 1;

void set_last_error(const std::string& s);
int cuda_fail(cudaError_t e, const char* what);
// Count of kernels this library has launched (cmm_launch_count).
void note_launch(int n = 1);
long long launch_count();

struct DeviceBuffer {
  void* p = nullptr;
  size_t bytes = 0;
  ~DeviceBuffer();
  int alloc(size_t n);
  int upload(const void* src, size_t n);
  void release();
};

}  // namespace cmm

struct cmm_mesh {
  cmm::MeshView view;
  cmm::DeviceBuffer verts, tri_v, tri_loc, tri_asm, root, root_f, root_adj, node_n, node_nf, leaf_row,
      status, theta, phi, grid, cos_theta, tri_asm_f, tri_loc_f, sh_ab, sh_fm, walk_f, walk_d, jump, ring_n,
      diag_n;
};

namespace cmm {
// kernels (locate.cu)
int launch_locate(const MeshView& m, const double* q, int64_t n, int32_t* tri, double* bcc,
                  cudaStream_t s);
struct BveState;
// st != NULL: write into st->vel[0] instead of coeffs.
int launch_assemble(const MeshView& m, const double* jets, int ncomp, double* coeffs,
                    cudaStream_t s, const BveState* st = nullptr);
// FP32 velocity records (rec32) from FP32 jets into st->vel[0].
int launch_assemble_f32_jets(const MeshView& m, const float* jets, cudaStream_t s, const BveState* st);
int launch_compose(const MeshView& m, const double* const* coeffs, int S, const double* q,
                   int64_t n, double* out, int32_t* tri, int32_t* tri_all, double* jac,
                   cudaStream_t s, const int32_t* perm = nullptr, const double* const* forms = nullptr,
                   const float* const* forms_ff = nullptr);
// Map-form records (Nt, kFormStride) from coefficient records (Nt, 64).
int launch_assemble_forms(const MeshView& m, const double* coeffs, double* forms, cudaStream_t s);
// Float-float form records (Nt, kFormFFStride) of form records.
int launch_forms_ff(const MeshView& m, const double* forms, float* forms_ff, cudaStream_t s);
// The forms of the stack slot a device-driven step remaps into (no-op on
// the other steps).
struct BveState;
int launch_remap_forms(const MeshView& m, const BveState* st, int n_maps, int Nt, const double* const* table,
                       double* const* ftable, cudaStream_t s);
// Query order by coarse cell (cmm_query_order): perm (n) and work
// (order_workspace(n) int32).
int64_t order_workspace(int64_t n);
int launch_query_order(const MeshView& m, const double* q, int64_t n, int32_t* perm, int32_t* work,
                       cudaStream_t s);
// Composition through the st->nc submaps of the device table `table`
// (submap 0 first) followed by `last` (applied first), no Jacobian.
int launch_compose_dev(const MeshView& m, const double* const* table, const BveState* st,
                       const double* last, const double* q, int64_t n, double* out, cudaStream_t s,
                       const double* const* ftable = nullptr);
int launch_stencil_eval(const MeshView& m, const double* coeffs, const double* yn,
                        const double* st, int64_t nv, double* out, cudaStream_t s);
// Host-side tables of an icosahedral mesh (before upload).
struct HostMesh {
  int level = 0, nv = 0, nt = 0;
  std::vector<double> vpad, loc, asmf, root, node_n, walk_d;
  std::vector<float> node_nf, walk_f;
  std::vector<int4> tv;
  std::vector<int> root_adj, leaf_row;
};
// Cube-map jump table of the walk location (maps.cu): every cell centre
// located by the hierarchy descent.
int build_jump_table(cmm_mesh* m);
int build_host(const double* verts, int nv, const int32_t* tris, int nt, int level, HostMesh* hm);
int upload_mesh(const HostMesh& h, cmm_mesh* m);
const char* last_error();

// lat-lon velocity mesh (velmesh.cpp) and kernels (velocity.cu)
int build_latlon(int L, const double* theta, const double* phi, const double* grid,
                 const double* verts, cmm_mesh* m);
void latlon_triangles(int L, std::vector<int4>& tv);

// Lagrange weights of the velocity time levels for up to 4 evaluation
// times (one per integrator stage).
struct TimeWeights {
  double w[4][3];
};
struct VelPtrs {
  const double* p[3];
};
TimeWeights time_weights(int nvs, double ts0, double dt, const double* times, int ntimes);
// Evaluation times of an integrator's stages (transport.cu); 0 = unknown.
int stage_times(int scheme, double t, double dt, double* times);

// Analytic transport flows and tracers (transport.cu); m is the map mesh
// (status word only for the point kernels).
int flow_velocity(const MeshView& m, int kind, double T, double alpha, double t, const double* x, int64_t n,
                  double* out, cudaStream_t s);
int flow_integrate(const MeshView& m, int kind, double T, double alpha, int scheme, double t, double dt,
                   const double* x, int64_t n, double* out, cudaStream_t s);
int flow_advect_points(const MeshView& mesh, int kind, double T, double alpha, int scheme, double t, double dt,
                       const double* s_pts, double* work, cudaStream_t s);
int launch_tracer(const MeshView& m, int kind, double t, const double* X, int64_t n, double* out,
                  cudaStream_t s);

// Device-resident state of a device-driven barotropic step (stepper.cu):
// read by the kernels of a step in place of their host arguments, so one
// captured CUDA graph replays every step; updated at the end of each step
// by bve_advance_kernel.
struct BveState {
  double* vel[3];   // velocity coefficient slots, oldest first
  TimeWeights tw;   // Lagrange weights of the next step's four RK4 stages
  double ts0;       // time of the oldest velocity level
  double step;      // tspan step (= dt)
  int k;            // tspan index of the next step's start time
  int count;        // steps taken (the driver's counter)
  int nc;           // submaps in the stack
  int identity;     // current map is the identity (right after a remap)
};
int launch_velocity_eval(const MeshView& vm, VelPtrs vc, int nvs, const TimeWeights& tw,
                         const double* x, int64_t n, double* out, cudaStream_t s);
int launch_integrate(const MeshView& vm, VelPtrs vc, int nvs, const TimeWeights& tw, int scheme,
                     double dt, const double* x, int64_t n, double* out, cudaStream_t s);
int launch_latlon_locate(const MeshView& vm, const double* q, int64_t n, int32_t* tri, double* bcc,
                         cudaStream_t s);
// st != NULL: velocity slots and stage weights from st (advect), the
// previous map dropped when st->identity (project).
int launch_advect_points(const MeshView& mesh, const MeshView& vm, VelPtrs vc, int nvs,
                         const TimeWeights& tw, int scheme, double dt, const double* s_pts,
                         double* work, cudaStream_t s, const BveState* st = nullptr);
int launch_project_jets(const MeshView& mesh, const double* prev_coeffs, const double* yn,
                        const double* sn, const double* tan, double eps, double* jets,
                        cudaStream_t s, const BveState* st = nullptr);

// Allocation-free variant of the map update (velocity.cu): foot-point
// scratch in a fixed device array sized for kNoAllocMaxVerts vertices.
constexpr int kNoAllocMaxVerts = 10242;
int advect_project_noalloc(const MeshView& mesh, const MeshView& vm, VelPtrs vc, int nvs,
                           const TimeWeights& tw, int scheme, double dt, const double* s_pts,
                           const double* tan, const double* prev_coeffs, double eps,
                           double* jets, cudaStream_t s);

int launch_vorticity(int kind, const double* params, int nparams, const double* sh, int lmax,
                     const MeshView& vm, const double* spline, double rot, const double* X,
                     int64_t Q, int npr, const double* cos_ring, double* omega, cudaStream_t s);


// adjoints (adjoint.cu)
constexpr int kAdjMaxSubmaps = 256;
int launch_assemble_bwd(const MeshView& m, const double* gc, double* gj, cudaStream_t s);
int launch_compose_bwd(const MeshView& m, const double* const* cs, double* const* gcs, int S,
                       const double* q, int64_t n, const double* gout, double* gq, double* work,
                       cudaStream_t s);
int launch_vorticity_bwd(const MeshView& vm, const double* dsh, int lmax, double rot, const double* X,
                         int64_t Q, const double* gw, double* gX, double* gsh, cudaStream_t s);
// work: cmm_advect_workspace (15 nv) + 12 nv doubles
int launch_advect_project_bwd(const MeshView& mesh, const MeshView& vm, const double* const* vel,
                              double* const* gvel, int nvs, const TimeWeights& tw, int scheme, double dt,
                              const double* s_pts, const double* tan, const double* prev, double* gprev,
                              double eps, const double* gjets, double* work, cudaStream_t s);
// FP32 copy of a mesh's factor table (velmesh records in FP32).
int make_asm_f32(cmm_mesh* m);

// spherical-harmonic transforms (sht.cu)
int sht_create(int L, cmm_sht** out);
int sht_destroy(cmm_sht* p);
int sht_L(const cmm_sht* p);
int sht_forward(cmm_sht* p, const double* samples, double2* out, cudaStream_t s);
int sht_inverse(cmm_sht* p, const double2* alm, int nf, double* samples, cudaStream_t s);
int sht_velocity(cmm_sht* p, const cmm_mesh* vm, const double* omega, double2* psi_out,
                 double* jets, cudaStream_t s);
// sht_velocity(p, vm, omega, NULL, jets) around a batch's analysis
int sht_velocity_pre(cmm_sht* p, const double* omega, cudaStream_t s);
int sht_velocity_post(cmm_sht* p, const cmm_mesh* vm, double* jets, cudaStream_t s);
int sht_batch_create(cmm_sht* const* plans, int n, cmm_sht_batch** out);
int sht_batch_destroy(cmm_sht_batch* bt);
int sht_batch_size(const cmm_sht_batch* bt);
// The split form's last velocity jets as floats (12 x Nv_u), or NULL.
const float* sht_jets_f32(const cmm_sht* p);
int sht_batch_analysis(cmm_sht_batch* bt, double2* const* out, cudaStream_t s);
int sht_batch_forward(cmm_sht_batch* bt, const double* const* samples, double2* const* alm, cudaStream_t s);
int sht_scalar_jets(cmm_sht* p, const cmm_mesh* vm, const double2* alm, double* jets, cudaStream_t s);
int sht_power(cmm_sht* p, const double2* alm, double* power, cudaStream_t s);
int* sht_status_word(cmm_sht* p);
int sht_set_tables(cmm_sht* p, int mode);
int sht_share_tables(cmm_sht* p, cmm_sht* src);
int sht_velocity_bwd(cmm_sht* p, const cmm_mesh* vm, const double* gjets, double* gomega, cudaStream_t s);
int sht_trim(cmm_sht* p);
int bve_create(const cmm_bve_desc* d, cmm_bve** out);
int bve_step(cmm_bve* b, cudaStream_t s);
int bve_step_pre(cmm_bve* b, cudaStream_t s);
int bve_step_post(cmm_bve* b, cudaStream_t s);
int bve_destroy(cmm_bve* b);
int bve_state(cmm_bve* b, cudaStream_t s, int* count, int* nc, int* identity);
int sht_set_precision(cmm_sht* p, int mode);
int sht_status(cmm_sht* p, cudaStream_t s, int* flags, int clear);

// split-BF16 tensor-core Legendre synthesis (sht_tc.cu)
// Upload per-triangle factors (nt, kAsmStride) factor-major (kAsmFactors, nt).
int upload_asm_factors(DeviceBuffer& dst, const std::vector<double>& asmf, int nt);

struct TcPlan;
int tc_plan_create(int L, const double* ct_rings, const double* pmm_rings, const double* ct_fine,
                   const double* pmm_fine, const double* ra, const double* rb, TcPlan** out);
void tc_plan_destroy(TcPlan* p);
int tc_plan_share(const TcPlan* src, TcPlan** out);
size_t tc_plan_bytes(const TcPlan* p);
int tc_synthesis(TcPlan* p, const double2* fields, float2* S, int* status, cudaStream_t s);
void tc_set_schedule(TcPlan* p, int schedule);
int sht_set_schedule(cmm_sht* p, int schedule);
int tc_analysis(TcPlan* p, const float2* fine, const double* w, double2* alm, int* status,
                cudaStream_t s);
// The analysis in two parts, for several fields of one band-limit sharing
// each streamed Pbar tile: the data tiles of one field into column pair
// `slot` of the 16-column tiles xtab (tc_xtab_bytes, zeroed by the owner),
// then the contraction of n <= 8 fields (slots 0..n-1) -> alm[b].
size_t tc_xtab_bytes(const TcPlan* p);
int tc_analysis_tiles(TcPlan* p, const float2* fine, const double* w, unsigned char* xtab, int slot,
                      cudaStream_t s);
int tc_analysis_batch(TcPlan* p, const unsigned char* xtab, double2* const* alm, int n, int* status,
                      cudaStream_t s);
int tc_wait_timeout_probe(long long polls, int* status, cudaStream_t s);
}  // namespace cmm
