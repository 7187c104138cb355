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

int cmm_mesh_create(const double* verts, int nv, const int32_t* tris, int nt, int level,
                    cmm_mesh** out) {
  if (!verts || !tris || !out) return arg_error("cmm_mesh_create: null pointer");
  *out = nullptr;
  cmm_mesh* m = new (std::nothrow) cmm_mesh();
  if (!m) return arg_error("cmm_mesh_create: out of host memory");
  int rc = set_split_tables();
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
  return launch_locate(mesh->view, q, n, tri, bcc, (cudaStream_t)stream);
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

int cmm_stencil_eval(const cmm_mesh* mesh, const double* coeffs, const double* yn,
                     const double* st, int64_t nv, double* out, void* stream) {
  if (!mesh || !coeffs || !yn || !st || !out || nv < 0)
    return arg_error("cmm_stencil_eval: bad argument");
  return launch_stencil_eval(mesh->view, coeffs, yn, st, nv, out, (cudaStream_t)stream);
}

}  // extern "C"
