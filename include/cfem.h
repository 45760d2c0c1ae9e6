/*
 * cfem.h -- C-ABI of the GB300 (sm_103a) element-by-element elasticity library.
 *
 * The reference (moarseniy/CudaFEMproject) exposes its path as C++ free
 * functions over a DEVICE_NAME switch (FEMproject/femfunc/src/femfunc.h:20-24)
 * plus the ElementsData / Matrix factories
 * (FEMproject/fem_utils/include/fem_utils_cpu.h:24-148,
 *  FEMproject/matrix_pack/include/matrix_pack_cpu.h:31-121). This header is the
 * flat boundary those calls map onto: plain pointers and sizes, status codes,
 * no C++ or torch types. The C++ mirror of the reference interface
 * (include/cfem_femfunc.hpp) and the Python driver both sit on top of it.
 *
 * Conventions
 *  - Every call returns a cfem_status; nothing exits the process (the reference
 *    calls exit() on assertion and NaN, Tools.cpp:27-33 / femfunc.cpp:107-110).
 *    cfem_last_error_string() gives the message of the last failure.
 *  - Vectors (displacements, right-hand sides) are in the caller's node order,
 *    DIM values per node, like dataKeeper::get_displacements()
 *    (datakeeper.cpp:64-66). Unless stated otherwise an array argument may be
 *    host memory or device memory of the context's GPU (copied with
 *    cudaMemcpyDefault on the context's stream).
 *  - One context per stream; no global mutable state besides the per-thread
 *    error string (replaces the reference's static cuBLAS handle,
 *    cuda_matrix.cpp:3-8) and the one device scratch array shared by all
 *    calls of cfem_matvec_energy_noalloc (see there).
 */
#ifndef CFEM_H
#define CFEM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CFEM_ABI_VERSION 1

#if defined(__GNUC__)
#define CFEM_API __attribute__((visibility("default")))
#else
#define CFEM_API
#endif

typedef enum cfem_status {
  CFEM_OK = 0,
  CFEM_ERR_INVALID_ARGUMENT = 1,
  CFEM_ERR_CUDA = 2,
  CFEM_ERR_OUT_OF_MEMORY = 3,
  CFEM_ERR_NOT_CONVERGED = 4,  /* iteration cap reached before the stopping rule */
  CFEM_ERR_DIVERGED = 5,       /* NaN / Inf in the PCG scalars (reference: exit(-1)) */
  CFEM_ERR_MESH = 6,           /* inconsistent mesh (bad ids, unused nodes, zero volume) */
  CFEM_ERR_UNSUPPORTED = 7,
  CFEM_ERR_IO = 8
} cfem_status;

/* Semantics of the numerical path. */
typedef enum cfem_semantics {
  CFEM_COMPAT = 0,     /* reproduce the reference's results, quirks included */
  CFEM_CONSISTENT = 1  /* textbook operators, masses and loads */
} cfem_semantics;

typedef enum cfem_precision {
  CFEM_FP64 = 0,         /* FP64 vectors and FP64 element operator */
  CFEM_FP32 = 1,         /* FP32 vectors and operator, FP64 reductions */
  CFEM_FP32_REFINE = 2   /* FP32 inner PCG inside FP64 iterative refinement */
} cfem_precision;

typedef enum cfem_stop_rule {
  CFEM_STOP_REFERENCE = 0, /* gamma_new < tol * gamma0, gamma = r.M^-1.r (femfunc.cpp:92) */
  CFEM_STOP_RESIDUAL = 1   /* ||r||_2 <= tol * ||f||_2 */
} cfem_stop_rule;

typedef enum cfem_matvec_form {
  CFEM_FORM_AUTO = 0,      /* edge fans in 3D, per element in 2D */
  CFEM_FORM_GRADIENT = 1,  /* stored scaled shape gradients: K_e p = G^T D G p, one thread per element */
  CFEM_FORM_STORED_KE = 2, /* stored 12x12 / 6x6 FP32 K_e (the reference's Klocals) */
  CFEM_FORM_GRADIENT_FAN = 3, /* gradient form, one thread per edge fan of up to 6 tets (3D) */
  CFEM_FORM_GEOMETRY_FAN = 4  /* edge fans; the FP32 matvec forms the gradients from streamed
                                 patch-relative coordinates instead of reading stored ones (3D) */
} cfem_matvec_form;

typedef enum cfem_wavelet_type { CFEM_WAVELET_NONE = 0, CFEM_WAVELET_RICKER = 1, CFEM_WAVELET_BERLAGE = 2 } cfem_wavelet_type;

/* The content of one prepared-mesh task (datakeeper.cpp:116-213). */
typedef struct cfem_mesh {
  int32_t dim;                   /* 2: CST triangles (plane stress), 3: linear tetrahedra */
  int64_t n_nodes;
  const double *nodes;           /* [n_nodes][dim] */
  int64_t n_elems;
  const int32_t *elems;          /* [n_elems][dim+1] 0-based node ids */
  int64_t n_constraints;
  const int32_t *constraints;    /* [n_constraints][2] node, Constraint::Type code (femstruct.h:39-52) */
  int64_t n_loads;
  const int32_t *load_nodes;     /* [n_loads] */
  const double *load_vectors;    /* [n_loads][dim] */
  int64_t n_faces;
  const int32_t *face_nodes;     /* [n_faces][dim+1] dim face nodes, then the opposite node */
  const int32_t *face_elems;     /* [n_faces] adjacent element */
  const double *face_normals;    /* [n_faces][dim] as in stress.txt (normalised internally) */
  const double *face_pressures;  /* [n_faces] */
  const double *elem_young;      /* [n_elems] per-element Young's modulus, or NULL */
} cfem_mesh;

typedef struct cfem_material {
  double young_modulus;  /* run_config youngModulus (default 2e7) */
  double poisson_ratio;  /* run_config poissonRatio (default 0.3) */
  double rho;            /* run_config rho (default 2400) */
} cfem_material;

typedef struct cfem_options {
  int32_t semantics;     /* cfem_semantics */
  int32_t matvec_form;   /* cfem_matvec_form */
  int32_t patch_elems;   /* elements per CTA patch, 0 = default (768 for edge fans, 512 per element);
                            cfem_autotune_patch_elems measures the best value for a mesh */
  int32_t verbose;       /* print PCG scalars like PRINT_DEBUG_INFO */
} cfem_options;

typedef struct cfem_wavelet {
  int32_t type;          /* cfem_wavelet_type */
  double freq, timeshift, ampl;
} cfem_wavelet;

typedef struct cfem_solve_params {
  int32_t precision;     /* cfem_precision */
  int32_t stop_rule;     /* cfem_stop_rule (inner rule for CFEM_FP32_REFINE) */
  double tol;            /* reference: 1e-8 static, 1e-4 dynamics. CFEM_FP32_REFINE: the inner FP32 PCG's
                            residual drop per refinement step; from 0.2 up the inner PCG keeps its search
                            direction across the FP64 true-residual replacements (fastest near 0.3-0.4),
                            below 0.2 each step restarts it */
  int32_t max_iter;      /* PCG iteration cap (per inner solve) */
  double outer_tol;      /* CFEM_FP32_REFINE: stop when ||f - K x||_2 <= outer_tol ||f||_2, or (for an
                            outer_tol below what FP64 can reach) when two refinement steps in a row no
                            longer reduce the FP64 true residual; info.rel_residual reports where it ended */
  int32_t max_outer;     /* CFEM_FP32_REFINE: refinement step cap */
} cfem_solve_params;

typedef struct cfem_solve_info {
  int32_t status;        /* cfem_status of the solve */
  int32_t iterations;    /* total PCG iterations (all inner solves) */
  int32_t outer_iterations;
  double rel_residual;   /* ||f - K x||_2 / ||f||_2, FP64 true residual */
  double gamma0, gamma;  /* first and last r.M^-1.r of the (last) PCG */
  double solve_ms;       /* device time of the solve (CUDA events) */
  int64_t kernel_launches; /* kernels issued by the solve (graph nodes included) */
} cfem_solve_info;

typedef struct cfem_dyn_params {
  double beta1, beta2;   /* GN22 parameters; explicit when beta2 == 0 (femfunc.cpp:145) */
  double dt, endtime;    /* steps = int(float(endtime) / float(dt)); endtime < 0: one relaxation step */
  int32_t precision;     /* CFEM_FP64 or CFEM_FP32 */
  double pcg_tol;        /* implicit: 1e-4 in compat (reference rule), else per stop_rule */
  int32_t stop_rule;
  int32_t max_iter;
  int32_t warm_start;    /* implicit: start each PCG from the previous acceleration */
  int32_t n_receivers;   /* optional trace recording: nodes and output buffer */
  const int32_t *receiver_nodes;
  double *receiver_trace; /* [steps][n_receivers][dim] displacements, host or device */
} cfem_dyn_params;

typedef struct cfem_dyn_info {
  int32_t status;
  int32_t steps;
  int64_t pcg_iterations;
  double solve_ms;
} cfem_dyn_info;

typedef struct cfem_ctx cfem_ctx;

/* ---- lifetime ---------------------------------------------------------- */
/* dataKeeper + ElementsData::setElementsData + genMask + calculateKlocals
 * (datakeeper.cpp:246-252, fem_utils.cpp:41-51, cpu_fem_utils.cpp:182-520):
 * uploads the mesh, renumbers it for locality, builds the DOF map, constraint
 * masks, element operators and right-hand sides. `stream` is a cudaStream_t
 * (NULL = legacy default stream). */
CFEM_API cfem_status cfem_create(cfem_ctx **ctx, const cfem_mesh *mesh, const cfem_material *mat,
                        const cfem_options *opt, void *stream);
CFEM_API void cfem_destroy(cfem_ctx *ctx);
CFEM_API const char *cfem_last_error_string(void);
CFEM_API int32_t cfem_abi_version(void);
CFEM_API cfem_status cfem_set_stream(cfem_ctx *ctx, void *stream);
CFEM_API cfem_status cfem_synchronize(cfem_ctx *ctx);
/* counts[0..5] = dim, n_nodes, n_elems, n_dof, n_patches, matvec_form */
CFEM_API cfem_status cfem_get_counts(const cfem_ctx *ctx, int64_t *counts);

/* ---- setup products, for bit-exact checks (host outputs) --------------- */
/* genMask (cpu_fem_utils.cpp:182-213): mask[e*w + dim*a + d] = dim*elem[e][a] + d, w = 6(dim-1). */
CFEM_API cfem_status cfem_dof_map(const cfem_ctx *ctx, int32_t *mask);
/* genAdjElements (cpu_fem_utils.cpp:215-219): elements touching each DOF. */
CFEM_API cfem_status cfem_adjacency(const cfem_ctx *ctx, int32_t *adj);
/* ParseConstraints (datakeeper.cpp:139-171): 1 for every constrained DOF. */
CFEM_API cfem_status cfem_bc_mask(const cfem_ctx *ctx, uint8_t *constrained);
/* Locality renumbering: new->old node and element permutations. */
CFEM_API cfem_status cfem_renumbering(const cfem_ctx *ctx, int32_t *node_new2old, int32_t *elem_new2old);
/* calculateKlocals + applyConstraints (cpu_fem_utils.cpp:489-520): row-major
 * w x w element matrices of elements [first, first+count) in the caller's order,
 * rebuilt in FP64 from the stored operator. */
CFEM_API cfem_status cfem_element_matrices(cfem_ctx *ctx, int64_t first, int64_t count, double *ke);
/* Assembled diagonal of the constrained stiffness (getDiagonal + reduction). */
CFEM_API cfem_status cfem_diagonal(cfem_ctx *ctx, double *diag);
/* initFlocals / calcFlocals at time t, assembled (cpu_fem_utils.cpp:522-596). */
CFEM_API cfem_status cfem_rhs(cfem_ctx *ctx, const cfem_wavelet *w, double t, double *f);

/* ---- operators and solvers --------------------------------------------- */
/* y = K' x, K' the constrained stiffness (Matrix::bmm + reductionWithMask,
 * femfunc.cpp:66-67 then assembly). precision CFEM_FP64: double x, y;
 * CFEM_FP32: float x, y. */
CFEM_API cfem_status cfem_matvec(cfem_ctx *ctx, int32_t precision, const void *x, void *y);
/* gpuPCG_EbE_vec (femfunc.cpp:25-128): Jacobi PCG for K' u = f from u = 0. */
CFEM_API cfem_status cfem_pcg(cfem_ctx *ctx, const cfem_solve_params *prm, const double *f, double *u, cfem_solve_info *info);
/* gpuCalculateFEM_EbE_vec (femfunc.cpp:3-23): static solve with the mesh's own loads. */
CFEM_API cfem_status cfem_static_solve(cfem_ctx *ctx, const cfem_wavelet *w, const cfem_solve_params *prm, double *u,
                              cfem_solve_info *info);
/* gpuCalculateFEM_DYN (femfunc.cpp:130-381): GN22 time stepping, final displacements. */
CFEM_API cfem_status cfem_dyn(cfem_ctx *ctx, const cfem_dyn_params *prm, const cfem_wavelet *w, double *u,
                     cfem_dyn_info *info);
/* k load cases at once: F, U are [k][n_dof] (RHS-major). The element operator
 * is streamed once per matvec for all k. info may be NULL or [k]. */
CFEM_API cfem_status cfem_pcg_multi(cfem_ctx *ctx, const cfem_solve_params *prm, int32_t k, const double *F, double *U,
                           cfem_solve_info *info);
/* Adjoint of the static solve K' u = f: lambda = K'^-1 dL/du, then
 * dL/dE_e = -lambda_e^T (dK'_e/dE_e) u_e and dL/df = lambda. Outputs may be NULL. */
CFEM_API cfem_status cfem_adjoint(cfem_ctx *ctx, const cfem_solve_params *prm, const double *u, const double *dLdu,
                         double *dLdE, double *dLdf, cfem_solve_info *info);
/* The whole reference flow for one task of a run_config file (main.cpp:18-33
 * with argv): read the config and the prepared mesh, run the static or dynamic
 * solve per task_type, optionally write results.vtk (VTKfile.cpp:281-386) into
 * <working_path>/fem_results/<DIM>D/<task>/. u_out (n_out doubles, may be NULL)
 * receives the displacements. Keys under "gb300" select precision/semantics. */
CFEM_API cfem_status cfem_run_task(const char *config_path, const char *task, int32_t write_vtk, double *u_out,
                                   int64_t n_out, cfem_solve_info *static_info, cfem_dyn_info *dyn_info);
/* results.vtk of given data (host only, no GPU), in the layout of the
 * reference's MakeVTKfile2D / MakeVTKfile3D (VTKfile.cpp:281-386): points
 * (printed as float), cells, cell types, displacement vectors and their
 * magnitudes. nodes [n_nodes][dim], elems [n_elems][dim + 1] (0-based),
 * u [n_nodes][dim] in FP32 like the reference's displacement matrix. */
CFEM_API cfem_status cfem_write_vtk(const char *path, int32_t dim, const double *nodes, int64_t n_nodes,
                                    const int32_t *elems, int64_t n_elems, const float *u);
/* Batched independent meshes (no counterpart in the reference, which solves
 * one mesh per process): n 3D meshes, each with its own material, in one
 * context. Node, element, constraint, load and face arrays are each mesh's
 * own (0-based per mesh); the batch concatenates them instance after instance
 * (cfem_batch_info gives the offsets). Only cfem_batch_static_solve and the
 * structural queries accept such a context; CFEM_ERR_UNSUPPORTED otherwise. */
/* ---- LS-DYNA keyword (.k) meshes (host only, no GPU) --------------------
 * The reference's converter (mesh_parser_lib/parser_src/parser_lib.py:36-378)
 * turns a keyword file into the prepared-mesh files; cfem_kfile_read reads the
 * same content into arrays: nodes [n][dim] (file order), elements [e][dim+1]
 * (0-based node positions), constraints [c][2] (node, constraint code),
 * nodal loads (node, [dim] vector), pressure faces ([dim+1]: the face's nodes,
 * then the element's remaining node; element; normal [dim], not normalised,
 * pointing away from the element; pressure). */
typedef struct cfem_kfile cfem_kfile;
CFEM_API cfem_status cfem_kfile_read(const char *path, int32_t dim, cfem_kfile **out);
CFEM_API cfem_status cfem_kfile_sizes(const cfem_kfile *k, int64_t *n_nodes, int64_t *n_elems, int64_t *n_constraints,
                                      int64_t *n_loads, int64_t *n_faces);
/* Copies the arrays into caller buffers sized by cfem_kfile_sizes (NULL skips one). */
CFEM_API cfem_status cfem_kfile_get(const cfem_kfile *k, double *nodes, int32_t *elems, int32_t *constraints,
                                    int32_t *load_nodes, double *load_vectors, int32_t *face_nodes, int32_t *face_elems,
                                    double *face_normals, double *face_pressures);
CFEM_API void cfem_kfile_free(cfem_kfile *k);

CFEM_API cfem_status cfem_create_batch(cfem_ctx **out, int32_t n, const cfem_mesh *meshes, const cfem_material *mats,
                                       const cfem_options *opt, void *stream);
/* (n <= 8192 instances) */
/* n instances; node_off / elem_off (may be NULL) receive n + 1 offsets into
 * the concatenated caller order. */
CFEM_API cfem_status cfem_batch_info(const cfem_ctx *ctx, int32_t *n, int64_t *node_off, int64_t *elem_off);
/* Static solve of every instance under its own loads, all instances in the
 * same kernel launches with per-instance PCG scalars and stopping tests (a
 * converged instance is skipped). prm->precision CFEM_FP32 or CFEM_FP32_REFINE
 * (per-instance FP64 refinement). u: concatenated displacements (n_dof of all
 * instances); info: NULL or [n]. */
CFEM_API cfem_status cfem_batch_static_solve(cfem_ctx *ctx, const cfem_solve_params *prm, double *u,
                                             cfem_solve_info *info);
/* Measurement: n back-to-back launches of the PCG-form matvec kernel (direction
 * update + element operator + scatter + p.Ap reduction) on the context's stream,
 * timed with CUDA events. Returns the mean device time per launch and the
 * algorithmic DRAM bytes of one launch: per element the stored operator and
 * local connectivity, per node z and p read, p written, y accumulated. */
CFEM_API cfem_status cfem_profile_matvec(cfem_ctx *ctx, int32_t precision, int32_t n_launches, double *ms_per_launch,
                                         double *bytes_per_launch);
/* Autotuner for the elements per CTA patch (no counterpart in the reference):
 * builds the mesh's context once per candidate patch size (NULL candidates:
 * 192, 384, 576, 768 tets for edge fans, 256, 512, 1024 elements otherwise),
 * times the FP32 PCG-form matvec of each on the current device, and returns
 * the fastest in *best (pass it as cfem_options.patch_elems).
 * ms_per_launch: NULL or [n_candidates] measured times. The cases-per-thread
 * parameter of cfem_pcg_multi is tuned inside that call. */
CFEM_API cfem_status cfem_autotune_patch_elems(const cfem_mesh *mesh, const cfem_material *mat, const cfem_options *opt,
                                               const int32_t *candidates, int32_t n_candidates, int32_t *best,
                                               double *ms_per_launch);
/* Element strains and stresses of a displacement field u (caller order):
 * strain = B u_e, stress = D_e strain in Voigt order (xx, yy, xy) / (xx, yy, zz,
 * xy, yz, xz), engineering shear; von Mises stress per element
 * (deprecated/femfunc/femfunc.cpp:42-106). Outputs [n_elems][3(dim-1)] or
 * [n_elems], caller element order; any output may be NULL. */
CFEM_API cfem_status cfem_element_stress(cfem_ctx *ctx, const double *u, double *strain, double *stress, double *mises);
/* Explicit GN22 (beta2 == 0, FP64, consistent semantics) receiver-misfit loss
 * L = 1/2 sum_{n=1..N} sum_r |d_n[node_r] - obs[n-1][r]|^2 and its gradient in
 * the per-element Young's moduli by the discrete adjoint of the time stepping.
 * The reverse sweep recomputes forward states segment by segment from
 * checkpoints stored every ceil(sqrt(N)) steps. obs: [N][n_rec][dim]. */
CFEM_API cfem_status cfem_dyn_adjoint(cfem_ctx *ctx, const cfem_dyn_params *prm, const cfem_wavelet *w, int32_t n_rec,
                                      const int32_t *rec_nodes, const double *obs, double *loss, double *dLdE,
                                      cfem_dyn_info *info);
/* y = K' x and *energy = x.K'x for callers that cannot allocate device memory:
 * code that runs inside another framework's memory pool (an allocator that owns
 * the whole device), or in a loop that must not hit the implicit device-wide
 * synchronisation of cudaMalloc / cudaFree. This call allocates nothing: x and
 * y are the caller's device arrays ([n_nodes][dim] FP64, caller node order),
 * energy points to one double in host or device memory (may be NULL), and the
 * only scratch is a fixed array compiled into the library (per-block partial
 * sums for at most CFEM_NOALLOC_MAX_BLOCKS blocks, about 33 KB, held on every
 * GPU that loads the library until the process exits). A context that needs
 * more blocks is rejected with CFEM_ERR_INVALID_ARGUMENT. The first call on a
 * device resolves the scratch address there. The call is synchronous: it
 * waits for its own work on the context's stream before it returns (so that a
 * host energy pointer holds the result), and so it cannot be recorded into a
 * CUDA graph by stream capture. All calls share the one scratch array, so
 * calls that overlap on the GPU (other streams, other threads, other
 * contexts) race and must be serialised by the caller. This entry point has no
 * counterpart in the reference. */
#define CFEM_NOALLOC_MAX_BLOCKS 4096
CFEM_API cfem_status cfem_matvec_energy_noalloc(cfem_ctx *ctx, const double *x, double *y, double *energy);
/* Self-test of the failure path of the FP32 edge-fan matvec's bulk copies
 * (3D single-mesh contexts): runs one matvec in which the first block of patch
 * 0 is never requested and the copy waits give up after ~1 ms, and checks
 * that the kernel flags the missing copy, returns, and the host reports it as
 * CFEM_ERR_CUDA ("a bulk copy ... did not complete in time"). Returns CFEM_OK
 * when all of that happened; the context stays usable. No GPU fault is
 * involved: the waits are bounded and nothing is read from the missing
 * block. Has no counterpart in the reference (its GPU path has no bulk
 * copies). */
CFEM_API cfem_status cfem_selftest_copy_timeout(cfem_ctx *ctx);
/* Per-element Young's modulus update (keeps geometry; rebuilds operator scale). */
CFEM_API cfem_status cfem_set_young(cfem_ctx *ctx, const double *elem_young);

#ifdef __cplusplus
}
#endif
#endif /* CFEM_H */
