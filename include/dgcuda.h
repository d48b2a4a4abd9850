/*
 * dgcuda.h - C ABI of the GB300 RK4 right-hand side for the linearised-Euler /
 * acoustic DG solver (drop-in for the step loop of DGFEM-Acoustic).
 *
 * What it replaces (reference file:line):
 *   dg_create      Mesh::precomputeMassMatrix (src/Mesh.cpp:440-466) and the
 *                  per-stage scratch set-up of solver::rungeKutta
 *                  (src/solver.cpp:173-194); it reads the arrays the Mesh
 *                  constructor builds (include/Mesh.h:31-108, 140-223).
 *   dg_set_state   the caller-owned state u[4][numNodes]
 *                  (src/dgalerkin.cpp:36, layout include/Mesh.h:34-36).
 *   dg_set_sources source node selection (src/solver.cpp:197-210).
 *   dg_rk4_steps   one iteration of the time loop per step: hard sources
 *                  (src/solver.cpp:248-256), the four RK stages of
 *                  Mesh::updateFlux (src/Mesh.cpp:569-674), numStep
 *                  (src/solver.cpp:35-52) with Mesh::precomputeFlux
 *                  (src/Mesh.cpp:500-539), Mesh::getElFlux (src/Mesh.cpp:548-557),
 *                  Mesh::getElStiffVector (src/Mesh.cpp:476-489), and the RK
 *                  combination (src/solver.cpp:261-285); t += dt.
 *   dg_get_state   the copy-out at save steps (src/solver.cpp:226-235);
 *                  dg_get_state_async / dg_wait_state overlap it with the
 *                  next steps.
 *   dg_monitors    no counterpart: FP64 discrete energy, L2 norms, NaN check.
 *   dg_error_vs    no counterpart: FP64 relative L2 error between two states.
 *
 * Conventions: 0 = success, negative = error (DG_ERR_*); no exceptions cross
 * the ABI.  A context is not thread-safe; use one per host thread.  The host
 * keeps ownership of every array passed in; dg_create copies what it needs.
 * Element and face data are passed at the first quadrature point; meshes
 * with curved (non-affine, isoparametric) elements also pass the reference's
 * per-quadrature-point arrays (the el_num_int_pts block of dg_mesh_desc).
 */
#ifndef DGCUDA_H
#define DGCUDA_H

#ifdef __cplusplus
extern "C" {
#endif

#define DG_OK 0
#define DG_ERR_ARG (-1)
#define DG_ERR_CUDA (-2)
#define DG_ERR_UNSUPPORTED (-3)
#define DG_ERR_NONFINITE (-4)
#define DG_ERR_IO (-5)
#define DG_ERR_MESH (-6)
#define DG_ERR_NOMEM (-7)
#define DG_ERR_CONFIG (-8)

#define DG_PREC_FP64 0 /* FP64 throughout */
#define DG_PREC_FP32 1 /* FP32 state, flux and geometry factors */
#define DG_PREC_MIXED 2 /* FP32 stage data, state kept as an FP32 pair, volume + lift
                         * contraction on the tensor cores (BF16 fixed-point slices,
                         * exact FP32 accumulation); orders 1-4 in 3D, 1-5 in 2D */
#define DG_PREC_TF32X3 3 /* as DG_PREC_MIXED, the contraction by 3xTF32 split products
                          * (a_hi b_hi + a_hi b_lo + a_lo b_hi, kind::tf32 MMAs, FP32
                          * accumulation); orders 1-4 in 3D, 1-5 in 2D */

#define DG_FLUX_REFERENCE 0 /* interior jump sign fc*orientation, as the reference (Mesh.cpp:524) */
#define DG_FLUX_UPWIND 1    /* interior jump sign +1 on every face */

typedef struct dg_ctx dg_ctx;

/* The reference Mesh arrays (include/Mesh.h), at the first quadrature point. */
typedef struct dg_mesh_desc {
    int dim;          /* m_elDim: 2 or 3 */
    int order;        /* m_elOrder: 1..5 */
    int num_el;       /* m_elNum */
    int el_num_nodes; /* m_elNumNodes */
    int f_num;        /* m_fNum */
    int f_num_per_el; /* m_fNumPerEl */
    int f_num_nodes;  /* m_fNumNodes */
    int fc;           /* numerical flux coefficient fc (Mesh.h:143, Mesh.cpp:210-211) */
    const double *el_jacobians;      /* [num_el][9]: dx_x/du_u at [u*3+x] (Mesh.h:37-39) */
    const double *el_jacobian_dets;  /* [num_el] (Mesh.h:40-42) */
    const double *f_normals;         /* [f_num][3] after the boundary flip (Mesh.h:88-90, Mesh.cpp:336-353) */
    const double *f_jacobian_dets;   /* [f_num] (Mesh.h:70-72) */
    const int *el_f_ids;             /* [num_el][f_num_per_el] (Mesh.h:91-93) */
    const int *el_f_orientation;     /* [num_el][f_num_per_el], +-1 (Mesh.h:100-102) */
    const int *f_nbr_el_ids;         /* [f_num][2], -1 for a missing side (Mesh.h:94-96) */
    const int *f_n_to_el_n_ids;      /* [f_num][f_num_nodes][2], -1 for a missing side (Mesh.h:97-99) */
    const int *f_bc;                 /* [f_num]: 1 reflecting, otherwise absorbing (Mesh.h:218) */
    const unsigned char *f_is_boundary; /* [f_num] (Mesh.h:217) */
    /* Curved elements: the per-point arrays of the reference Mesh on its
     * Gauss(2p) rules (Mesh.cpp:31-38, 135-194).  Zero / NULL for meshes of
     * straight-sided elements.  An element whose Jacobian differs between its
     * points (relative 1e-11) runs the per-point (curved) form; every other
     * element runs the affine form on its first-point data. */
    int el_num_int_pts;                  /* m_elNumIntPts */
    const double *el_int_param_coords;   /* [Ng][4] u, v, w, weight (m_elIntParamCoords) */
    const double *el_basis_fcts;         /* [Ng][Np] (m_elBasisFcts, Mesh.h:46-48) */
    const double *el_ugrad_basis_fcts;   /* [Ng][Np][3] (m_elUGradBasisFcts) */
    const double *el_jacobians_qp;       /* [num_el][Ng][9] dx_x/du_u at [u*3+x] (m_elJacobians, Mesh.h:37-39) */
    const double *el_jacobian_dets_qp;   /* [num_el][Ng] (m_elJacobianDets) */
    int f_num_int_pts;                   /* m_fNumIntPts */
    const double *f_int_param_coords;    /* [Ngf][4] (m_fIntParamCoords) */
    const double *f_basis_fcts;          /* [Ngf][Nfp] (m_fBasisFcts, Mesh.h:85-87) */
    const double *f_normals_qp;          /* [f_num][Ngf][3] after the boundary flip (m_fNormals, Mesh.h:88-90) */
    const double *f_jacobian_dets_qp;    /* [f_num][Ngf] (m_fJacobianDets) */
} dg_mesh_desc;

/* Mean flow and medium (include/configParser.h:26-28). */
typedef struct dg_phys_desc {
    double c0, rho0;
    double v0[3];
} dg_phys_desc;

typedef struct dg_opts {
    int precision;   /* DG_PREC_FP64 | DG_PREC_FP32 | DG_PREC_MIXED | DG_PREC_TF32X3 */
    int flux_sign;   /* DG_FLUX_REFERENCE | DG_FLUX_UPWIND */
    int device;      /* CUDA device ordinal */
    int use_graph;   /* capture step chunks in CUDA graphs (1) or launch directly (0) */
    int elems_per_block; /* 0 = built-in choice */
    int tc_pipelines;    /* tensor-core forms: independent tile pipelines per CTA,
                          * 0 or 1 = one, 2 = two where tensor and shared memory
                          * allow (else one; dg_tc_info tells) */
    int reserved[2];
} dg_opts;

/* Per-kernel timing of dg_profile_steps (CUDA events on the solver stream). */
typedef struct dg_kernel_times {
    double stage_ms[4];   /* summed device time of the (affine) stage kernels */
    int stage_launches[4];
    double inject_ms;
    int inject_launches;
    double total_ms;      /* first event to last event */
    double curved_ms;     /* summed device time of the curved-element stage kernel */
    int curved_launches;
} dg_kernel_times;

void dg_default_opts(dg_opts *opts);

int dg_create(const dg_mesh_desc *mesh, const dg_phys_desc *phys, const dg_opts *opts, dg_ctx **out);
void dg_destroy(dg_ctx *ctx);

/* u[q] points to num_el*el_num_nodes doubles, field q = p, vx, vy, vz,
 * element-major (u[q][el*el_num_nodes + n]).  In 2D vz must be zero. */
int dg_set_state(dg_ctx *ctx, const double *const u[4]);
int dg_get_state(dg_ctx *ctx, double *const u[4]);

/* Asynchronous copy-out for save steps (replaces the blocking copy of
 * src/solver.cpp:226-235 at each timeRate): the state of member 0, as it is
 * after the work already enqueued, is snapshotted in FP64 on the solver
 * stream and copied to host[4*num_el*el_num_nodes] (fields p, vx, vy, vz one
 * after the other; vz = 0 in 2D) on a side stream, so the following steps
 * run while the frame crosses the host link.  Returns at once with a ticket;
 * dg_wait_state(ticket) blocks until that frame is in host.  host must stay
 * valid until then, and should be pinned (dg_host_alloc) for the copy to
 * overlap: a pageable buffer makes the call wait for the copy.  Two frames
 * can be in flight; a third call first waits for the oldest. */
int dg_get_state_async(dg_ctx *ctx, double *host, long long *ticket);
int dg_wait_state(dg_ctx *ctx, long long ticket);

/* Staged state upload (the counterpart of dg_get_state_async for a caller
 * that feeds a new state every step): dg_stage_state starts the copy of
 * host[4*num_el*el_num_nodes] (fields p, vx, vy, vz one after the other; vz
 * is ignored in 2D and not checked) into a device staging buffer on a side
 * stream and returns at once with a ticket; dg_commit_state(ticket) makes
 * that copy the state of member 0, in stream order: after the work already
 * enqueued (the steps before it see the old state) and before any work
 * enqueued later.  A stage called before the previous step lets the copy
 * cross the host link while that step runs.  host must stay unchanged until
 * the commit has run (a later dg_rk4_steps, dg_get_state or dg_synchronize
 * returns after it), and should be pinned (dg_host_alloc) for the copy to
 * overlap.  Two staged states can wait; a third stage reuses the oldest
 * slot (committing an overwritten ticket is DG_ERR_ARG). */
int dg_stage_state(dg_ctx *ctx, const double *host, long long *ticket);
int dg_commit_state(dg_ctx *ctx, long long ticket);

/* Hard sources: for source s, nodes dof_idx[offsets[s] .. offsets[s+1]) get
 * p = amp*sin(2*pi*freq*t + phase) while t < duration, at the start of each
 * step.  params[s*4 + 0..3] = amp, freq, phase, duration.  Later sources
 * overwrite earlier ones on shared nodes.  In a batch context every member
 * gets the same sources. */
int dg_set_sources(dg_ctx *ctx, int nsrc, const int *offsets, const int *dof_idx, const double *params);

/* Batch contexts (no counterpart in the reference, which runs one source
 * configuration per process): nbatch independent states on one mesh, stepped
 * together by every step call (one launch per stage covers all members).
 * dg_create is dg_create_batch with nbatch = 1.  dg_set_state sets every
 * member, dg_get_state and dg_monitors read member 0. */
int dg_create_batch(const dg_mesh_desc *mesh, const dg_phys_desc *phys, const dg_opts *opts, int nbatch,
                    dg_ctx **out);
int dg_set_state_member(dg_ctx *ctx, int member, const double *const u[4]);
int dg_get_state_member(dg_ctx *ctx, int member, double *const u[4]);

/* Per-member sources: source s acts on member[s] only, node k of it with
 * p = weights[k]*amp*sin(2*pi*freq*t + phase) (weights may be NULL: all 1,
 * the reference's hard source).  Replaces any earlier source set. */
int dg_set_batch_sources(dg_ctx *ctx, int nsrc, const int *member, const int *offsets, const int *dof_idx,
                         const double *weights, const double *params);

/* Receivers: after every step the pressure of every member at nrec nodes is
 * recorded on the device, for the first max_steps steps after this call.
 * dg_get_traces copies out[member][rec][max_steps] and the number of steps
 * recorded. */
int dg_set_receivers(dg_ctx *ctx, int nrec, const int *dof_idx, int max_steps);
int dg_get_traces(dg_ctx *ctx, double *out, int *steps);

/* nsteps classical RK4 steps starting at *t; *t is advanced by repeated
 * t += dt in double, as the reference loop does. */
int dg_rk4_steps(dg_ctx *ctx, double *t, double dt, int nsteps);

/* nsteps forward-Euler steps starting at *t (sources, then u += dt*RHS(u)),
 * the loop body of solver::forwardEuler (src/solver.cpp:138-153), selected by
 * timeIntMethod = Euler1 (src/dgalerkin.cpp:55-56; the reference's default). */
int dg_euler_steps(dg_ctx *ctx, double *t, double dt, int nsteps);

/* dg_rk4_steps bracketed by CUDA events on the solver stream; *ms = device
 * time of the whole run. */
int dg_rk4_steps_timed(dg_ctx *ctx, double *t, double dt, int nsteps, double *ms);

/* Same steps with CUDA events around every kernel (no graph). */
int dg_profile_steps(dg_ctx *ctx, double *t, double dt, int nsteps, dg_kernel_times *times);

/* FP64 monitors: energy = 1/2 sum_e u_e^T M_e (p^2/(rho0 c0^2) + rho0 |v|^2);
 * l2[q] = sqrt(u_q^T M u_q); status = number of non-finite values (the call
 * then returns DG_ERR_NONFINITE).  The mixed form's state is read as the FP64
 * sum of its FP32 pair. */
int dg_monitors(dg_ctx *ctx, double *energy, double *l2, long long *status);

/* FP64 error monitor (no counterpart in the reference, whose only monitor is
 * a progress line, solver.cpp:240-244): rel_l2[q] = ||u_q - r_q|| / ||r_q||
 * over the nodal values of field q, for member `member` of ctx against member
 * `ref_member` of ref, two contexts on the same mesh and device, of any
 * precision (FP32 pairs joined in FP64).  Accumulated in FP64 on the device;
 * only the 8 sums cross to the host.  Waits for ref's stream, then enqueues
 * on ctx's and waits.  rel_l2[q] = 0 for fields the mesh does not evolve;
 * *status (may be null) = non-finite values in ctx's state, DG_ERR_NONFINITE
 * when nonzero. */
int dg_error_vs(dg_ctx *ctx, int member, dg_ctx *ref, int ref_member, double *rel_l2, long long *status);

/* Waits for all work of the context. */
int dg_synchronize(dg_ctx *ctx);

/* Sizes and the device data the context holds (for callers that time or
 * inspect it): number of DOFs per field, fields evolved, bytes of state. */
int dg_info(dg_ctx *ctx, long long *dofs_per_field, int *fields, long long *state_bytes);

/* Tensor-core forms: tile pipelines per CTA of the context's stage kernels
 * and elements per tile (both 0 for the FP64 and FP32 forms). */
int dg_tc_info(dg_ctx *ctx, int *pipelines, int *tile_elems);

/* Curved elements of the context (run by the per-point kernel) and the
 * points of the element and face rules they use. */
int dg_curved_info(dg_ctx *ctx, int *ncurved, int *points, int *face_points);

/* Pinned host buffers for fast dg_set_state / dg_get_state. */
void *dg_host_alloc(unsigned long long bytes);
void dg_host_free(void *p);

/* Host-side view of the element-centric layout dg_create uploads (no GPU
 * work; for inspection and tests).  geo [num_el][dim*dim] inverse Jacobians
 * B[x][u]; fgeo [num_el][nf][4] outward normal and detJf/detJe; conn
 * [num_el][nf][2] neighbour and connectivity word (bits 0-1 neighbour's local
 * face, 2-4 face permutation, 5-6 kind 0 interior / 1 reflecting /
 * 2 absorbing, 7 negative jump sign); ops = D as [u][j][i] then LIFT as
 * [face*nfp+k][i]; tabs = face masks [nf][nfp] then permutations
 * [nperm][nfp]; mass [np][np] reference mass matrix. */
typedef struct dg_layout dg_layout;
typedef struct dg_layout_view {
    int dim, order, np, nf, nfp, nq, nperm, num_el;
    const double *geo;
    const double *fgeo;
    const int *conn;
    const double *ops;
    int n_ops;
    const unsigned char *tabs;
    int n_tabs;
    const double *mass;
} dg_layout_view;
int dg_layout_build(const dg_mesh_desc *mesh, int flux_sign, dg_layout **out);
int dg_layout_get(const dg_layout *layout, dg_layout_view *view);
void dg_layout_free(dg_layout *layout);

/* RK4 steps that allocate no device memory (no counterpart in the reference).
 *
 * For callers that must not call cudaMalloc: code inside an application that
 * hands all device memory out of its own pool (a private cudaMalloc would
 * fail once the pool has taken the memory, or fragment it), and time loops
 * that cannot afford the implicit device synchronisation an allocation or a
 * free may cause.  The caller
 * owns every array it passes: the FP64 device layout (the arrays
 * dg_layout_build returns, copied to the device) and the state u (device,
 * [dim+1][num_el*np], field-major, updated in place).  The three RK4 stage
 * buffers live in one fixed device array inside the library, 24 MiB, which
 * every GPU that loads the library holds until the process exits; states of
 * more than 1,048,576 values (fields x element nodes) are rejected with
 * DG_ERR_UNSUPPORTED.  Work is enqueued on `stream` (a cudaStream_t, 0 for
 * the default stream) and not waited for; *t advances by dt per step.
 * Every call looks up the array's device address in the current device's
 * context (cudaGetSymbolAddress, which allocates nothing), so a device that
 * the application reset is served at the array's new address; the first
 * call on a device loads the library's kernels into that context, so make
 * it before any stream capture.  Alignment: fgeo 16 bytes, conn, geo, ops
 * and u 8 bytes (cudaMalloc and pool allocations of 256-byte granularity
 * satisfy both); other pointers are refused with DG_ERR_ARG before any
 * launch.  All calls share the one array, which keeps the previous call's
 * contents (nothing in it needs to start at zero): calls whose work
 * overlaps on the GPU race on it. */
typedef struct dg_device_layout {
    int dim, order, num_el;
    double c0, rho0, v0[3];
    const double *geo;          /* device [num_el][dim*dim] */
    const double *fgeo;         /* device [num_el][nf][4] */
    const int *conn;            /* device [num_el][nf][2] */
    const double *ops;          /* device, D then LIFT as in dg_layout_view */
    const unsigned char *tabs;  /* device face masks then permutations */
} dg_device_layout;
int dg_rk4_steps_noalloc(const dg_device_layout *layout, double *u, double *t, double dt, int nsteps, void *stream);

/* Uneven multi-mesh batches (no counterpart in the reference, which runs one
 * mesh per process): nmesh 3D meshes of any sizes and orders 1-5, each with
 * its own medium and mean flow, stepped together by one persistent launch
 * per RK4 stage (a list of (mesh, element tile) work items shared by the
 * CTAs), or one per order present (configuration 3), chunks of steps
 * captured in CUDA graphs.  FP64 or FP32.  Every mesh
 * has its own time t[i] and step dt[i]. */
typedef struct dg_multi dg_multi;
int dg_multi_create(int nmesh, const dg_mesh_desc *meshes, const dg_phys_desc *phys, const dg_opts *opts,
                    dg_multi **out);
void dg_multi_destroy(dg_multi *ctx);
int dg_multi_set_state(dg_multi *ctx, int mesh, const double *const u[4]);
int dg_multi_get_state(dg_multi *ctx, int mesh, double *const u[4]);
/* Sources as dg_set_batch_sources, with a mesh index per source. */
int dg_multi_set_sources(dg_multi *ctx, int nsrc, const int *mesh, const int *offsets, const int *dof_idx,
                         const double *weights, const double *params);
int dg_multi_rk4_steps(dg_multi *ctx, double *t, const double *dt, int nsteps);
int dg_multi_rk4_steps_timed(dg_multi *ctx, double *t, const double *dt, int nsteps, double *ms);
/* Configurations: 0-2 make one persistent launch per stage for all meshes
 * with CTAs of block_threads[k] threads (elements per CTA = block threads /
 * element nodes for each order); 3 (block_threads 0) makes one persistent
 * launch per order present, each with the CTA size and shared memory of the
 * single-mesh kernels of that order.  dg_multi_autotune times each on
 * trial_steps steps of the batch (the state is restored), keeps the fastest
 * and reports ms per step of every candidate. */
int dg_multi_set_config(dg_multi *ctx, int cfg);
int dg_multi_autotune(dg_multi *ctx, const double *dt, int trial_steps, int *chosen, double *ms_per_step);
int dg_multi_info(dg_multi *ctx, long long *dofs_per_field, int *ncfg, int *cfg, int *block_threads);

/* Learned coarse propagator and parareal (no counterpart in the reference).
 *
 * dg_mlp: a fully connected network nin -> width (GELU) x hidden_layers ->
 * nout in FP32, trained on the GPU by its own forward, backward (mean
 * squared error) and Adam kernels.  Parameters are packed per layer as the
 * weights [out][in] row-major followed by the biases [out]. */
typedef struct dg_mlp dg_mlp;
int dg_mlp_create(int nin, int width, int nout, int hidden_layers, unsigned seed, int device, dg_mlp **out);
void dg_mlp_destroy(dg_mlp *net);
long long dg_mlp_num_params(const dg_mlp *net);
int dg_mlp_get_params(dg_mlp *net, float *params);
int dg_mlp_set_params(dg_mlp *net, const float *params);
/* X [rows][nin] -> Y [rows][nout] (host arrays). */
int dg_mlp_forward(dg_mlp *net, const float *X, int rows, float *Y);
/* The same inference on the tcgen05 tensor cores: inputs, weights and hidden
 * activations rounded to BF16 (weights refreshed whenever the FP32 master
 * weights change), FP32 accumulation, bias and GELU in FP32; layers of at
 * most 256 outputs (DG_ERR_UNSUPPORTED otherwise). */
int dg_mlp_forward_bf16(dg_mlp *net, const float *X, int rows, float *Y);
/* Mean squared error over rows x nout against T and its gradient (packed
 * like the parameters; grad may be NULL). */
int dg_mlp_loss_grad(dg_mlp *net, const float *X, const float *T, int rows, double *loss, float *grad);
int dg_mlp_train_step(dg_mlp *net, const float *X, const float *T, int rows, double lr, double *loss);
/* Where the GEMMs of training (forward pass, activation and weight
 * gradients) run: 1 = the tcgen05 tensor cores with 3xTF32 split products
 * and FP32 accumulation (the default), 0 = the CUDA cores (FP32 FMA).  FP32
 * inference (dg_mlp_forward, FP32 coarse steps) runs on the CUDA cores. */
int dg_mlp_set_gemm(dg_mlp *net, int mode);

/* dg_learned: an element-local network (inputs: the element's DOFs, its face
 * neighbours' traces at its face nodes, its boundary-face kinds and inverse
 * Jacobian; outputs: the element's DOF increments over coarse_steps fine RK4
 * steps of size dt) trained on FP64 DG trajectories of the mesh. */
typedef struct dg_learned dg_learned;
int dg_learned_create(const dg_mesh_desc *mesh, const dg_phys_desc *phys, int flux_sign, int width,
                      int hidden_layers, int coarse_steps, double dt, unsigned seed, int device, dg_learned **out);
void dg_learned_destroy(dg_learned *learned);
int dg_learned_info(dg_learned *learned, int *nin, int *nout, dg_mlp **net);
/* Runs the FP64 DG from u0 for nsnap x coarse_steps steps and keeps the
 * (features, increments) pairs of active elements, at most max_rows per
 * snapshot. */
int dg_learned_collect(dg_learned *learned, const double *const u0[4], int nsnap, int max_rows);
long long dg_learned_num_samples(dg_learned *learned);
int dg_learned_train(dg_learned *learned, int epochs, int batch, double lr, unsigned seed, double *loss);
/* Each coarse application adds alpha x the predicted increment, alpha <= 1
 * the largest factor that does not raise the discrete energy (lumped mass);
 * the number of applications so far and their mean and least alpha. */
/* Coarse steps infer with BF16 tensor cores (1) or FP32 (0, the default). */
int dg_learned_set_inference(dg_learned *learned, int bf16);
int dg_learned_step_stats(dg_learned *learned, long long *applications, double *alpha_mean, double *alpha_min);
/* napps coarse applications on a host state, in place. */
int dg_learned_apply(dg_learned *learned, double *const u[4], int napps);

/* Parareal over nslices time slices of slice_steps FP64 RK4 steps each from
 * u0: the fine propagator is the FP64 DG run for all slices as one batch,
 * the coarse one the learned network (slice_steps / coarse_steps
 * applications) or, with learned = NULL, the identity.  Stops when the
 * largest relative change of a slice end state is at most tol, or after
 * max_iter iterations (max_iter = nslices reproduces the serial DG).  uout
 * gets the end state of the last slice, hist[k] the change at iteration k. */
int dg_parareal(dg_learned *learned, const dg_mesh_desc *mesh, const dg_phys_desc *phys, int flux_sign,
                const double *const u0[4], int nslices, int slice_steps, double dt, double tol, int max_iter,
                double *const uout[4], int *iters, double *hist);

/* Message of the last error on this thread. */
const char *dg_last_error(void);

/* ---- Test hooks: not part of the drop-in surface. ----------------------
 * Exported so the GPU tests can exercise the tensor-core primitives and the
 * bounded-wait error path directly; an integration never calls them.
 *
 * dg_tc_selftest: a 128x32x112 BF16 GEMM with A in tensor memory and B in
 * shared memory on the given device; *max_abs_err = 0 when the FP32 result
 * is exact.
 * dg_tc_selftest_tf32: the same product with kind::tf32 MMAs (A as TF32
 * values in tensor memory, one per column; B in shared memory), exact.
 * dg_tc_wait_selftest: the same MMAs, then a 1 ms bounded wait on an
 * mbarrier that nothing arrives on.  The wait runs out and the kernel takes
 * the stage kernels' error path: it records the timeout (*flags bit 0),
 * drains its own MMAs with a second bounded wait (bit 1 set only if that
 * also runs out), frees its tensor memory and returns, leaving the context
 * usable.  Returns DG_OK when the kernel ran; *flags = 1 is the expected
 * outcome. */
int dg_tc_selftest(int device, double *max_abs_err);
int dg_tc_selftest_tf32(int device, double *max_abs_err);
int dg_tc_wait_selftest(int device, int *flags);

#ifdef __cplusplus
}
#endif
#endif /* DGCUDA_H */
