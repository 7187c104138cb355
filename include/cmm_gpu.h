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
  CMM_ERR_UNSUPPORTED = 7
} cmm_status;

/* Bits of the device status word. */
#define CMM_FLAG_NONFINITE 1
#define CMM_FLAG_LOCATE 2

const char* cmm_last_error(void);
int cmm_version(void);

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

/* Stencil evaluation: locate each vertex foot point yn[:,v] (3,nv), then
 * evaluate the 4 stencil foot points st (3,4,nv) in that same Powell-Sabin
 * sub-triangle, un-normalised -> out (3,4,nv).  Replaces
 * sphere_diffeomorphism.stencil_eval (cmm_s2/core/spherical_spline.py:268-298). */
int cmm_stencil_eval(const cmm_mesh* mesh, const double* coeffs, const double* yn,
                     const double* st, int64_t nv, double* out, void* stream);

#ifdef __cplusplus
}
#endif
#endif
