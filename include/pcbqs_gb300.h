/*
 * pcbqs_gb300 -- C ABI of the GB300 (sm_103a) static-fill and solve backend for pcbqs.
 *
 * Plain pointers and sizes only. Every function returns 0 on success or a status code:
 *   1 invalid argument, 2 CUDA error, 3 non-finite result, 4 device allocation failed,
 *   5 no convergence, 6 a bounded device wait gave up.
 * pcbqs_gb300_last_error() returns the calling thread's last message.
 *
 * "host" arguments are host memory; "device" arguments are device memory of the context's GPU. Entry points named
 * *_device take a CUDA stream (cudaStream_t, may be NULL for the legacy default stream) and are asynchronous on it
 * unless stated; the others are synchronous.
 *
 * Each declaration names the reference interface it replaces (paths within the pcbqs project).
 */
#ifndef PCBQS_GB300_H
#define PCBQS_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pcbqs_gb300_ctx pcbqs_gb300_ctx;

/* Host views of a prepared fill geometry: the arrays of FillGeometry (src/pcbqs/static_backends.py:94-130) and the
 * per-level observation rules of _offplane_geometry (src/pcbqs/_numerics/sing.py:56-69), row-major float64:
 * v (nt,3,2), len (nt,3), tau (nt,3,2), un (nt,3,2), area (nt), p3 (nt,3,2), cent (nt,2), radius (nt), z (nt);
 * qp[k] (nt,nq[k],2) and qw[k] (nq[k]) for k = 0, 1, 2 (a level that was not prepared may repeat level 0's). */
typedef struct pcbqs_gb300_geometry {
    int32_t nt;
    const double *v, *len, *tau, *un, *area, *p3, *cent, *radius, *z;
    const double *qp[3];
    const double *qw[3];
    int32_t nq[3];
} pcbqs_gb300_geometry;

/* Upload a geometry to `device` once and keep it resident. Replaces the device setup of a fill backend factory,
 * factory(FillGeometry, workers, chunk, device) (src/pcbqs/static_backends.py:268-270; the CuPy precedent
 * src/pcbqs/static_cupy.py:73-106). */
int pcbqs_gb300_create(const pcbqs_gb300_geometry *geometry, int device, pcbqs_gb300_ctx **ctx);
void pcbqs_gb300_destroy(pcbqs_gb300_ctx *ctx);
const char *pcbqs_gb300_last_error(void);
int32_t pcbqs_gb300_triangles(const pcbqs_gb300_ctx *ctx);
/* Kernels this library has launched in the process so far (for launch accounting). No reference counterpart. */
int64_t pcbqs_gb300_kernel_launches(void);
/* The solver keeps the device memory of its dense blocks, factors and Krylov bases in a stream-ordered pool after
 * each call, so that repeated solves reuse it; this returns the unused part of `device`'s pool to the device
 * (synchronizes the device). No reference counterpart. */
int pcbqs_gb300_release_memory(int device);
/* The near-pair counts of the context's last fill: counts[0] at level 0, counts[1] at the refined level. Their
 * sum is the analytic count static_fill reports (src/pcbqs/core/static_kernels.hpp:251). */
int pcbqs_gb300_fill_counts(const pcbqs_gb300_ctx *ctx, uint64_t *counts);

/* Pair protocol: moments of n ordered pairs (p observation, q source) at offsets d with quadrature kind
 * (-1 far, 0/1/2 analytic level), out (n, 1) if scalar_only else (n, 6) ordered M0, Mro_x, Mro_y, Mrs_x, Mrs_y,
 * Mrr; host arrays, returns after the results are in `out`. Replaces backend.evaluate(p, q, d, kind, scalar_only)
 * (src/pcbqs/static_backends.py:1-9, :300-336) and the compiled static_pairs
 * (src/pcbqs/core/static_kernels.hpp:147-172). Status 3 if a moment is not finite. */
int pcbqs_gb300_pairs(pcbqs_gb300_ctx *ctx, const int32_t *p, const int32_t *q, const double *d,
                      const int32_t *kind, int64_t n, int scalar_only, double *out);

/* The same on device arrays (p, q, d, kind, out), ordered on `stream`; synchronizes `stream` at the end to read
 * back the non-finite flag. */
int pcbqs_gb300_pairs_device(pcbqs_gb300_ctx *ctx, const int32_t *p, const int32_t *q, const double *d,
                             const int32_t *kind, int64_t n, int scalar_only, double *out, void *stream);

/* The same as pcbqs_gb300_pairs_device, for callers that cannot allow device allocation during a call (a
 * caching allocator already holds the device memory, or a steady-state loop must not stall in cudaMalloc or
 * cudaFree). It allocates nothing: its scratch is one fixed array in this library's device image, shared by every
 * call on a device, which limits a call to 1,048,576 pairs (larger n: status 1 with a message). The first call on
 * a device looks up that array's address there. Every call synchronizes `stream` and reads its status flags back
 * into host memory, so a call cannot be captured into a CUDA graph. Calls whose work overlaps on the GPU race on
 * the shared scratch: serialize them. Has no counterpart in the reference. */
int pcbqs_gb300_pairs_no_alloc(pcbqs_gb300_ctx *ctx, const int32_t *p, const int32_t *q, const double *d,
                               const int32_t *kind, int64_t n, int scalar_only, double *out, void *stream);

/* Whole reciprocal moment matrices into host planes (each nt x nt, row-major float64; planes[1..3] unused when
 * scalar_only): M0, Mx, My, Mrr with [p,q] = Mro, [q,p] = Mrs, the diagonal their average. near < 0 or infinite:
 * every pair analytic. *analytic receives the number of unordered pairs that were not far.
 * Replaces fill_symmetric(matrices, near, outer_levels, scalar_only) (src/pcbqs/static.py:35-42,
 * src/pcbqs/static_cupy.py:127-197) and the compiled static_fill (src/pcbqs/core/static_kernels.hpp:184-252). */
int pcbqs_gb300_fill(pcbqs_gb300_ctx *ctx, double near, int outer, int scalar_only, double *const *planes,
                     uint64_t *analytic);

/* The same into device planes of leading dimension ld >= nt; synchronizes `stream` at the end (it reads back the
 * near-pair counts and the non-finite flag). */
int pcbqs_gb300_fill_device(pcbqs_gb300_ctx *ctx, double near, int outer, int scalar_only, double *const *planes,
                            int64_t ld, uint64_t *analytic, void *stream);

/* Mixed precision: the same fill into FP32 planes holding moments about each triangle's centroid (Mx/My: the
 * centroid-relative Mro forward and Mrs reverse; Mrr the product of both offsets): far pairs integrated in FP32 in
 * these local coordinates, near pairs in FP64 and shifted to them. New in this backend (the reference fills FP64
 * only); its combine is pcbqs_gb300_edge_inductance_local_device. */
int pcbqs_gb300_fill_local_device(pcbqs_gb300_ctx *ctx, double near, int outer, int scalar_only, float *const *planes,
                                  int64_t ld, uint64_t *analytic, void *stream);

/* L = factor diag(scale) combine(moments) diag(scale), symmetric, from device moment planes (leading dimension
 * ldm) into device L (ne x ne, leading dimension ldl): tri (2,ne) int32 supports T+/T-, alpha (2,ne), vertex
 * (2,ne,2), scale (ne), all device arrays. Replaces the compiled static_combine
 * (src/pcbqs/core/static_kernels.hpp:257-310) behind static.edge_inductance (src/pcbqs/static.py:103-128). */
int pcbqs_gb300_edge_inductance_device(int64_t ne, const int32_t *tri, const double *alpha, const double *vertex,
                                       const double *scale, double factor, const double *mrr, const double *mx,
                                       const double *my, const double *m0, int64_t ldm, double *L, int64_t ldl,
                                       void *stream);

/* Host-array form of the same (static_combine's signature): moments (nt x nt) and L (ne x ne) on the host. */
int pcbqs_gb300_edge_inductance(int64_t nt, int64_t ne, const int32_t *tri, const double *alpha,
                                const double *vertex, const double *scale, double factor, const double *mrr,
                                const double *mx, const double *my, const double *m0, double *L);

/* Mixed precision combine (FP32 arithmetic, no cancellation) of the local moments of
 * pcbqs_gb300_fill_local_device: off (2,ne,2) holds centroid - free vertex of each support, alpha/off/scale FP32;
 * writes L (FP64, ldl) and, when Lf is not NULL, its FP32 copy (ldlf). Replaces static_combine for the mixed form. */
int pcbqs_gb300_edge_inductance_local_device(int64_t ne, const int32_t *tri, const float *alpha, const float *off,
                                             const float *scale, double factor, const float *mrr, const float *mx,
                                             const float *my, const float *m0, int64_t ldm, double *L, int64_t ldl,
                                             float *Lf, int64_t ldlf, void *stream);

/* P from FP32 M0 (the mixed fill), sums in FP64; Pf (NULL or an FP32 copy with the same row stride ldp). */
int pcbqs_gb300_potential_single_device(int64_t nn, const int64_t *start, const int32_t *members, const double *area,
                                        const float *m0, int64_t ldm, double factor, double *P, float *Pf,
                                        int64_t ldp, void *stream);

/* P = factor * W^T M0 W with W[t, a] = 1/area[a] for the triangles t of charge node a (members[start[a] ..
 * start[a+1])): device arrays; P (nn x nn, leading dimension ldp). factor = 1/(4 pi eps0 er).
 * Replaces MQS._set_potential (src/pcbqs/mqs.py:532-552). */
int pcbqs_gb300_potential_device(int64_t nn, const int64_t *start, const int32_t *members, const double *area,
                                 const double *m0, int64_t ldm, double factor, double *P, int64_t ldp,
                                 void *stream);

/* ---- H-matrix of L ----------------------------------------------------------------------------------------------
 * kind 0: L over RWG edges (below); kind 1: the potential kernel over triangles, factor M0(t,u) / (A_t A_u) with
 * factor = 1/(4 pi eps0 er) (PotentialEntries, src/pcbqs/core/hmatrix_build.hpp:54-67; the edge arrays are unused).
 * Blocks are described by meta (nblocks x 8 int64, device): a offset, a length, b offset, b length (into idx, the
 * edges of each cluster), store offset, rank cap, same (diagonal block), rank (written by the build: -1 dense,
 * >= 0 low rank). Edge arrays: tri (2,ne) int32 supports, alpha (2,ne) +-1/(2A), vertex (2,ne,2) centred; entries
 * factor * sum alpha alpha [Mrr - v.Mro - v.Mrs + v.v M0] of the canonical pair moments.
 * Build: the `dense` blocks get their la x lb entries (row-major at the store offset); the `lowrank` blocks get a
 * partial-pivot ACA (U la x cap column-major, V cap x lb, then 32 x lb check rows of scratch), rank cap as given,
 * accepted when 16 check rows and 16 independent ones are within tol; used: nlow x used_stride bytes of scratch.
 * Replaces the reference's level build (src/pcbqs/hmatrix.py:179-207 -> core/hmatrix_build.hpp:143-351 aca_blocks,
 * dense_blocks) with the RwgEntries provider (core/hmatrix_build.hpp:27-52, core/compressed_kernels.hpp:9-38). */
int pcbqs_gb300_hmatrix_build(const pcbqs_gb300_ctx *ctx, double near, int outer, int kind, const int32_t *tri,
                              const double *alpha, const double *vertex, int64_t ne, double factor, int64_t *meta,
                              const int64_t *dense, int64_t ndense, const int64_t *lowrank, int64_t nlow,
                              const int64_t *idx, double tol, double *store, unsigned char *used,
                              int64_t used_stride, void *stream);
/* Y = H X, X and Y (n, k) complex128 device arrays: each block writes its contributions into its slots (slot0:
 * nblocks x 2 int64, first slot of the a rows and of the transposed b rows), then every row sums its slots
 * (row_ptr (n+1), slots_of_row) in block order; slots: nslots x k complex128 scratch. Replaces HBlocks.apply
 * (src/pcbqs/core/hmatrix_kernels.hpp:20-100, packing src/pcbqs/hmatrix.py:234-297). */
int pcbqs_gb300_hmatrix_apply(int64_t n, int64_t nblocks, const int64_t *meta, const int64_t *slot0,
                              const int64_t *idx, const double *store, const int64_t *row_ptr,
                              const int64_t *slots_of_row, int max_rank, int k, const double *x, double *y,
                              double *slots, void *stream);

/* The PEEC loop basis on the host (src/pcbqs/mqs.py:48-130 spanning_tree, :592-637 _loops): branches k < nb
 * between nodes ea[k], eb[k] (is_src: current-source branches, never in the tree); the first `first` branches
 * (copper) form a breadth-first forest from each island's most central node, the other non-source branches only
 * join islands. tree_out (nb) marks the forest; every other branch (except copper inside one node when
 * ideal_terminals, and branches between islands) gets its fundamental cycle as COO entries (rows = branch,
 * cols = cycle index, vals = +-1) and col_branch[cycle] = its branch. Status 1 with *nnz = the entries needed when
 * capacity is short. No device work. */
int pcbqs_gb300_loop_basis(int64_t n_nodes, int64_t nb, const int32_t *ea, const int32_t *eb, const uint8_t *is_src,
                           int64_t first, int ideal_terminals, uint8_t *tree_out, int64_t capacity, int32_t *rows,
                           int32_t *cols, double *vals, int64_t *nnz, int32_t *col_branch, int64_t *ncol);

/* Layered-dielectric image sums (src/pcbqs/core/layered_kernels.hpp:38-120, layered_pairs) for every pair of
 * triangles p = rows[i], q = cols[j] (same != 0: the pairs rows[i], rows[j] with j >= i of one layer; cols unused),
 * written to both (p, q) and (q, p) of two FP64 planes, real and imaginary (ld >= triangles). Images: distances
 * ascending with the zero-distance images first, complex coefficients (interleaved re, im); spline (optional,
 * spline_m intervals, breaks x[0..m] from 0 to rho_max, coefficients [4][m] complex, highest power first) of the
 * smooth positive images. near < 0: every pair analytic. All arrays on the device; synchronizes `stream`. */
int pcbqs_gb300_layered_device(pcbqs_gb300_ctx *ctx, double near, int outer, const int32_t *rows, int64_t nrows,
                               const int32_t *cols, int64_t ncols, int same, const double *image_dist,
                               const double *image_coef, int nimages, const double *spline_x, const double *spline_c,
                               int64_t spline_m, double rho_max, double *out_re, double *out_im, int64_t ld,
                               void *stream);

/* ---- Biot-Savart near field --------------------------------------------------------------------------------
 * H at npts points (pts (npts,3) device, m) of sheet currents given as nsrc quadrature points src (nsrc,4: x,y,z,0)
 * with current moments jx, jy (nsrc, k) complex128 (w J_x, w J_y), accumulated into H (npts, 3, k) complex128;
 * single != 0 sums in FP32. Replaces biot._h_tris inside h_sheets (src/pcbqs/biot.py:24-79); the quadrature points
 * and the near refinement are built on the host as h_sheets builds them. */
int pcbqs_gb300_biot_sheets(int64_t npts, const double *pts, int64_t nsrc, const double *src_xyz4, const double *jx,
                            const double *jy, int k, int single, double *H, void *stream);
/* Straight filaments p0 -> p1 ((nseg,3) m) with currents I (nseg, k) complex128, accumulated into H. Replaces
 * biot.h_segments (src/pcbqs/biot.py:82-105). */
int pcbqs_gb300_biot_segments(int64_t npts, const double *pts, int64_t nseg, const double *p0, const double *p1,
                              const double *I, int k, double *H, void *stream);

/* Cloud-in-cell deposit of sheet-current moments onto a uniform grid (src/pcbqs/_numerics/currents.py:28-61,
 * current_deposit): point t at (qx[t], qy[t]) with complex moments mom_x, mom_y (npts, k, interleaved re, im) adds
 * its bilinear shares to jx, jy (nx, ny, k complex, row-major over x then y) at grid x0 + i dx, y0 + j dy; points
 * outside drop the shares that fall off the grid. Device arrays; the caller zeroes the grids and divides by the
 * cell area. Asynchronous on `stream`. */
int pcbqs_gb300_current_deposit(int64_t npts, const double *qx, const double *qy, const double *mom_x,
                                const double *mom_y, int k, double x0, double y0, double dx, double dy, int64_t nx,
                                int64_t ny, double *jx, double *jy, void *stream);

/* ---- Solve: the PEEC operator in loop/tree coordinates and batched GMRES ------------------------------------
 * Complex vectors of k systems are (n, k) row-major complex128 (interleaved re, im) device arrays. */

/* A sparse matrix in CSR form on the device: ptr (rows+1) int64, idx (nnz) int32, val (nnz) float64. */
typedef struct pcbqs_gb300_csr {
    int64_t rows, cols;
    const int64_t *ptr;
    const int32_t *idx;
    const double *val;
} pcbqs_gb300_csr;

/* The operator of peec_iterative.solve's product (src/pcbqs/peec_iterative.py:267-278) at nsys frequencies:
 *   out_s = K^T (R + j w_s L) K D_s y / zscale_s + T^T P T y / pscale,  D_s = diag(1 | j w_s zscale_s / pscale)
 * K (nb x n) the loop/tree basis over passive branches, Kt = K^T, T (nn x n) = A K restricted to the tree unknowns,
 * Tt = T^T, R (ne x ne) the copper's sparse resistance, L (ne x ne, row stride ldl) and P (nn x nn, ldp) dense
 * symmetric, is_tree (n) int8 marks the tree unknowns; omega and zscale are host arrays (nsys). The device arrays
 * must stay alive while the operator is used. */
typedef struct pcbqs_gb300_peec_desc {
    int64_t n, nb, ne, nn;
    pcbqs_gb300_csr K, Kt, T, Tt, R;
    const double *L;
    int64_t ldl;
    const double *P;
    int64_t ldp;
    const int8_t *is_tree;
    double pscale;
    int32_t nsys;
    const double *omega, *zscale;
    /* per system, the complex factor on R (interleaved re, im; null: 1): a finite-thickness sheet impedance
     * Zs(f) sigma t, so R(f) = rscale R (src/pcbqs/mqs.py:517-530, conductor.py:12-26) */
    const double *rscale;
    /* imaginary part of P (same leading dimension; null: P real), for a lossy dielectric stack */
    const double *Pim;
    /* rscale applies to the first nscaled rows of R (the sheets' edges) and not to the rest (plated via barrels,
     * which keep their DC resistance); 0: to every row. The preconditioners scale all of K^T R K (they need not be
     * exact); the operator is exact. */
    int64_t nscaled;
} pcbqs_gb300_peec_desc;

typedef struct pcbqs_gb300_peec pcbqs_gb300_peec;

/* Replaces the LinearOperator `product` of peec_iterative.solve (src/pcbqs/peec_iterative.py:267-278, 322). */
int pcbqs_gb300_peec_create(const pcbqs_gb300_peec_desc *desc, pcbqs_gb300_peec **op);
void pcbqs_gb300_peec_destroy(pcbqs_gb300_peec *op);
/* out = A_s in for k columns, column c at system sys[c] (host array); synchronizes `stream`. */
int pcbqs_gb300_peec_apply(pcbqs_gb300_peec *op, int k, const int32_t *sys, const double *in, double *out,
                           void *stream);
/* Block-Jacobi preconditioner on consecutive blocks of `bs` unknowns: krk (nblk, bs, bs) device array holds the
 * diagonal blocks of K^T R K; K^T L K and T^T P T blocks are gathered on the device; every (system, block) is
 * inverted. New in this backend: the reference preconditions with sparse surrogates
 * (src/pcbqs/peec_iterative.py:19-84, 283-321). */
int pcbqs_gb300_peec_block_jacobi(pcbqs_gb300_peec *op, int32_t bs, const double *krk, void *stream);
/* Single-precision direct preconditioner: the dense loop/tree system at system index sys, assembled on the device
 * (K^T L K and T^T P T formed once from the dense L and P; krk the sparse K^T R K as a device CSR n x n), in
 * complex64 and LU-factored. math 0: cuSOLVER getrf in FP32 arithmetic; math 1: cuSOLVER getrf, FP32 emulated with
 * BF16x9 products on the tensor cores (same FP32 accuracy); math 2 / 3: this library's blocked factorization
 * (pcbqs_gb300_lu_factor_c64, 2048-column panels) with BF16x9 / FP32 GEMMs. Mirrors MixedLU (src/pcbqs/kernels.py:125-181): a complex64 factor
 * with the FP64 operator's GMRES on top in place of its refinement loop. */
int pcbqs_gb300_peec_factor(pcbqs_gb300_peec *op, const pcbqs_gb300_csr *krk, int32_t sys, int math, void *stream);
/* A split of the graph Laplacian's kept rows into `parts` domains whose interiors share no edge, and a separator
 * (pcbqs_gb300_graph.domains). New order: the domains' interiors one after another, then the separator. dom_ptr
 * and bnd_ptr are HOST arrays, the rest device arrays. */
typedef struct pcbqs_gb300_graph_domains {
    int64_t parts;
    int64_t n_int;                 /* interior rows (the separator has nkeep - n_int) */
    const int64_t *perm;           /* nkeep: the kept row at each new position */
    const int64_t *pos;            /* nkeep: each kept row's new position */
    const int64_t *dom_ptr;        /* host, parts + 1: each domain's first new position (dom_ptr[parts] = n_int) */
    const int64_t *bnd_ptr;        /* host, parts + 1: each domain's first boundary entry */
    const int32_t *bnd;            /* per boundary entry: the separator node's position within the separator */
    const int64_t *bnd_nptr;       /* per boundary entry + 1: its interior neighbours in the domain */
    const int32_t *bnd_local;      /*   the neighbour's row within its domain */
    const int32_t *bnd_branch;     /*   the branch between them */
} pcbqs_gb300_graph_domains;
/* The graph preconditioner's structure and its values at one frequency (pcbqs_gb300_peec_graph); every pointer a
 * device array, complex values interleaved (re, im). Unknowns in the operator's order; "kept" nodes are all but one
 * grounded node per component, whose equation T[keep] drops. */
typedef struct pcbqs_gb300_graph {
    int64_t nkeep;                 /* kept nodes */
    int64_t ncomp;                 /* components of the passive branches' graph */
    int64_t nbranch;               /* passive branches (the length of zdiag, dinv) */
    pcbqs_gb300_csr ac;            /* nkeep x n: each loop's defining branch's incidence, +1 first end, -1 second */
    const int64_t *lap_ptr;        /* nkeep + 1: each kept node's passive branches (self-loops left out) */
    const int32_t *lap_branch;     /*   the branch */
    const int32_t *lap_other;      /*   its other end's kept row, -1 at a root */
    pcbqs_gb300_csr tinv;          /* n x nkeep: T[keep]^-1 (the spanning forest's path sums), rows of tree unknowns */
    pcbqs_gb300_csr tinvt;         /* nkeep x n: its transpose */
    const int32_t *branch;         /* n: each unknown's branch (a loop's defining branch, a tree unknown's own) */
    const int32_t *loop_ends;      /* n x 2: a loop's defining branch's ends as kept rows (-1 at a root) */
    const int32_t *comp;           /* nkeep: each kept node's component */
    const int64_t *member_ptr;     /* ncomp + 1 */
    const int32_t *members;        /* the kept rows of each component */
    const double *zdiag;           /* nbranch complex: each branch's own impedance r R_ii + j w L_ii */
    const double *dinv;            /* nbranch complex: 1 / zdiag, |zdiag| raised to 1e-12 zscale where smaller */
    const double *pinv;            /* nkeep complex: 1 / P_ii at the kept nodes */
    const double *total;           /* ncomp complex: the sum of 1 / P_ii over each component's nodes */
    const pcbqs_gb300_graph_domains *domains;   /* host struct, or NULL: the Laplacian dense */
} pcbqs_gb300_graph;
/* The reference's graph preconditioner (_graph_preconditioner and the charge-tree solve of _tree_preconditioner,
 * src/pcbqs/peec_iterative.py:19-84, without face-sheet pairs) at system index sys, for precondition 3 of
 * pcbqs_gb300_peec_gmres and pcbqs_gb300_peec_solve_mixed: the loop currents from the graph Laplacian
 * G = Ap diag(dinv) Ap^T [keep][:, keep] in place of the reference's sparse incomplete LU: domains NULL, G assembled
 * dense on the device and LU-factored in complex64 with this library's tcgen05 updates; else split into domains
 * (explicit complex64 inverses of their blocks, applied as GEMMs) and a dense Schur complement on the separator
 * (complex64 LU); `refine` (0..3) FP64 residual corrections of each Laplacian solve. The tree unknowns' charges
 * through the explicit T[keep]^-1 and the components' equilibrium. Works with the dense and the compressed
 * operator; the domain split's solves cannot be captured (captured GMRES cycles need domains NULL). The structure's
 * arrays must outlive the handle (the frequency's values are copied). Status 4 when the Laplacian's factors do not
 * fit in device memory, 3 when a factor meets a zero pivot. */
int pcbqs_gb300_peec_graph(pcbqs_gb300_peec *op, const pcbqs_gb300_graph *g, int32_t sys, int refine, void *stream);
/* out = M in for k columns (device, (n, k) complex128 row-major) with the graph preconditioner set up last
 * (validation of the preconditioner alone); synchronizes `stream`. */
int pcbqs_gb300_peec_graph_apply(pcbqs_gb300_peec *op, int k, const double *in, double *out, void *stream);
/* CUDA-event times (ms, on the factorization's stream) of the last pcbqs_gb300_peec_factor: the dense system's
 * assembly (with K^T L K and T^T P T when first formed) and the LU itself. No counterpart in the reference (its
 * factor is LAPACK on the host); for the roofline of the factorization. */
int pcbqs_gb300_peec_factor_times(const pcbqs_gb300_peec *op, double *assemble_ms, double *getrf_ms);
/* captured = 1: the GMRES of pcbqs_gb300_peec_gmres and of pcbqs_gb300_peec_solve_mixed (its inner solves) runs each
 * restart cycle as one CUDA graph launch: the Arnoldi steps in a conditional WHILE node whose condition a device
 * kernel sets (a column still active, steps left), each column's convergence mask on the device, no host
 * synchronization between steps; the graph is captured once per active-set size. The same kernels in the same
 * order as captured = 0 (the default: one host check per step), so the same results. The reference's batched
 * counterpart is mqs_iterative._lockstep_gmres (src/pcbqs/mqs_iterative.py:109-170), a host loop per step. */
int pcbqs_gb300_peec_set_captured(pcbqs_gb300_peec *op, int captured);
/* The inner products of pcbqs_gb300_peec_solve_mixed over 16 or more right-hand sides: terms = 3 (the default) or 6
 * BF16 parts on the tensor cores (pcbqs_gb300_dense_apply_tensor; L and P packed once after each
 * pcbqs_gb300_peec_single), 0 for the FP32 product throughout. The FP64 outer refinement sets the answer's accuracy
 * either way; the parts kept change the inner solves' work. No counterpart in the reference, whose inner products are
 * NumPy's (src/pcbqs/peec_iterative.py:253-256). */
int pcbqs_gb300_peec_set_product(pcbqs_gb300_peec *op, int terms);
/* The operator's FP64 dense products (pcbqs_gb300_peec_apply, the FP64 GMRES, the mixed solve's outer residuals)
 * over 4 or more right-hand sides: slices = 2..7 on the tensor cores (pcbqs_gb300_dense_apply_sliced; L and P sliced
 * once), 0 (the default) on the FP64 pipe. No counterpart in the reference, whose products are NumPy's FP64
 * (src/pcbqs/peec_iterative.py:253-256). */
int pcbqs_gb300_peec_set_fp64_product(pcbqs_gb300_peec *op, int slices);

/* An H-matrix as pcbqs_gb300.hmatrix.DeviceHMatrix packs it (the arrays of pcbqs_gb300_hmatrix_apply), device arrays;
 * nslots: the product's slot count. */
typedef struct pcbqs_gb300_hmat {
    int64_t n, nblocks, nslots;
    const int64_t *meta, *slot0, *idx, *row_ptr, *slots_of_row;
    const double *store;
    int32_t max_rank;
} pcbqs_gb300_hmat;
/* The compressed operator (the descriptor's L and P may then be null): L's first L->n rows (the RWG edges) from the
 * inductance H-matrix, the nv via segments after them from the dense block `via` (nv x nv, FP64, may be null when
 * nv = 0), and P = W^T H W from the triangle potential's H-matrix with W (triangles x nodes, A_t / A_node) and its
 * transpose Wt. Every product of the operator then goes through them (FP64); the complex64 factor and the mixed
 * solve need the dense matrices. Mirrors matrix_backend='hierarchical' (src/pcbqs/mqs.py:452-455; the products of
 * peec_iterative.py:267-278 through HMatrix._native_matmat and compressed.PotentialOperator, compressed.py:194-204). */
int pcbqs_gb300_peec_set_compressed(pcbqs_gb300_peec *op, const pcbqs_gb300_hmat *L, const double *via, int64_t nv,
                                    const pcbqs_gb300_hmat *P, const pcbqs_gb300_csr *W, const pcbqs_gb300_csr *Wt);
/* An H-matrix's low-rank blocks packed for the tensor cores by pcbqs_gb300.hmatrix.DeviceHMatrix.lowrank_plan
 * (device arrays): the dense blocks alone (meta_dense, slot0_dense: ndense records in the hmat's layout), the left
 * factors' plane (lrows x 128 BF16), the right factors' plane (128 x 2 rwidth BF16), the groups (one per block and
 * direction, 40-byte records: a_row0, rows, a_x0, b_x0, kb, t_row0, rank, pad as int32, slot0 as int64), the phase-two
 * tiles (ntiles pairs of group and row tile) and every row's position in the padded cluster order (n_pad wide). */
typedef struct pcbqs_gb300_lowrank {
    const int64_t *meta_dense, *slot0_dense;
    int64_t ndense;
    const void *lplane;
    int64_t lrows;
    const void *rplane;
    int64_t rwidth;
    const void *groups;
    int32_t ngroups, ntiles;
    const int32_t *tile_group, *tile_m, *pad_pos;
    int64_t n_pad;
    /* optional (dplane null: the dense leaves stay FP64): the dense leaves on the tensor cores, their plane
     * (drows x 2 dpitch BF16), groups and tiles in the same formats; meta_dense is then empty */
    const void *dplane;
    int64_t drows, dpitch;
    const void *dgroups;
    int32_t ndgroups, ndtiles;
    const int32_t *dtile_group, *dtile_m;
} pcbqs_gb300_lowrank;
/* Y = H X with the dense blocks in FP64 and the low-rank blocks' stacked U (V^T X) products on the tcgen05 tensor
 * cores: BF16 three-part products, FP32 accumulation (phase one R X[J] for every block and direction, one tile each;
 * phase two L T into the block's slots; the rows then sum their slots in block order). X, Y (n, k) complex128 device
 * arrays, k <= 128; relative error about 2^-16 of the low-rank part. Synchronizes `stream`; status 6 when a bounded
 * wait gave up. The reference's low-rank products are FP64 (core/hmatrix_kernels.hpp:20-100). */
int pcbqs_gb300_hmatrix_apply_lowrank(const pcbqs_gb300_hmat *H, const pcbqs_gb300_lowrank *lr, int k,
                                      const double *x, double *y, void *stream);
/* The BF16 part planes of pcbqs_gb300_lowrank from the H-matrix's FP64 store (device arrays; no counterpart in the
 * reference): jobs (njobs x 8 int64: base, si, sj, ni, nj, row0, colbase, map_off) each write the entries
 * x = store[base + i si + j sj], i < ni, j < nj, split as h = bf16(x), m = bf16(x - h) (x rounded to FP32, every
 * rounding to nearest even), to plane[(row0 + i) pitch + c] and plane[(row0 + i) pitch + off2 + c],
 * c = colbase + map[map_off + j] (colbase + j when map_off < 0); the jobs' destinations must not overlap. Ordered
 * on `stream`. */
int pcbqs_gb300_pack_bf16_parts(const double *store, const int64_t *jobs, int64_t njobs, const int32_t *map,
                                void *plane, int64_t pitch, int64_t off2, void *stream);
/* The compressed operator's single-precision view (the mixed solve's inner products): the H-matrix of L (which 0)
 * or of P (1) applied with its low-rank blocks on the tensor cores as pcbqs_gb300_hmatrix_apply_lowrank; the FP64
 * products (outer residuals) keep FP64 throughout. */
int pcbqs_gb300_peec_set_lowrank(pcbqs_gb300_peec *op, int which, const pcbqs_gb300_lowrank *lr);
/* Block-Jacobi (as pcbqs_gb300_peec_block_jacobi) from diagonal blocks the caller computed: klk and tpt (nblk, bs, bs)
 * device arrays of K^T L K and T^T P T (the compressed operator's, from exact entries). */
int pcbqs_gb300_peec_block_jacobi_blocks(pcbqs_gb300_peec *op, int32_t bs, const double *krk, const double *klk,
                                         const double *tpt, void *stream);
/* P x = b (nn x k complex128, device) by GMRES on the operator's own P products (dense or compressed) with the
 * Jacobi preconditioner diag (nn, device): the equilibrium charge of the compressed model (the dense model's is
 * pcbqs_gb300_dense_gmres). Status 5 when a column did not converge. */
int pcbqs_gb300_peec_potential_gmres(pcbqs_gb300_peec *op, int k, const double *b, double *x, const double *diag,
                                     double tol, int maxiter, int restart, int32_t *iterations, double *residual,
                                     void *stream);

/* The autotuner. Choices timed at first use are remembered per device (name and SM count) and problem size: the FP32
 * dense product's shape ("dense_f32 rows=R"), the triangular solves' method per column bucket ("trisolve n=N
 * columns=C": 0 streaming sweeps, 1 blocked) and the blocked LU's panel width ("lu_panel n=N math=M", timed only by
 * pcbqs_gb300_tune_lu_panel). pcbqs_gb300_tune_file sets a file (null or "": none) whose entries are merged in at
 * once and which is rewritten after every new choice; without a call, PCBQS_GB300_TUNE_FILE names it. No
 * counterpart in the reference (its solvers have no tunable shapes). */
int pcbqs_gb300_tune_file(const char *path);
/* The choice recorded for `key` on the current device; status 1 when none is. */
int pcbqs_gb300_tune_lookup(const char *key, int32_t *value);
/* Records a choice for `key` on the current device (as a timing would; e.g. to pin one by hand). */
int pcbqs_gb300_tune_record(const char *key, int32_t value);
int64_t pcbqs_gb300_tune_count(void);
void pcbqs_gb300_tune_clear(void);
/* Times pcbqs_gb300_lu_factor_c64's blocked factorization (math 0..3) of a synthetic diagonally dominant n x n
 * complex64 matrix with each panel width and records the fastest (*best) for pcbqs_gb300_peec_factor. Allocates
 * n^2 complex64 and synchronizes `stream`. */
int pcbqs_gb300_tune_lu_panel(int64_t n, int math, const int32_t *widths, int count, int32_t *best, void *stream);
/* The tcgen05 trailing updates of the last pcbqs_gb300_peec_factor with math 4 or 5: their summed CUDA-event time
 * (ms, on the factorization's stream), complex flops (8 rows cols k each) and count; zeros after any other math.
 * No counterpart in the reference; for the roofline of the update kernel. */
int pcbqs_gb300_peec_factor_updates(const pcbqs_gb300_peec *op, double *update_ms, double *update_flops,
                                    int32_t *launches);
/* Dense complex64 LU with partial pivoting of the n x n column-major device matrix a (leading dimension n), in
 * place, ipiv (device, n) receiving 1-based pivot rows: cusolverDnCgetrf's layout and pivots, so getrs and this
 * library's triangular solvers apply to it. Blocked: `block`-column panels (32 .. 4096) factored on a second stream
 * one step ahead of the trailing GEMMs; math 0: FP32 GEMMs (cuBLAS), 1: FP32 GEMMs emulated with BF16x9 on the
 * tensor cores (cuBLAS), 2 / 3: this library's tcgen05 update (pcbqs_gb300_complex_update) with 3 / 6 BF16 part
 * products, the subtraction fused into its epilogue. Returns status 6 if a bounded wait of that update gave up.
 * *singular (host) = 1-based index of the first exactly zero pivot, 0 if none. Synchronizes `stream`. The factor
 * step of MixedLU and lu_factor_rows (src/pcbqs/kernels.py:125-160, :266-285), which LAPACK's cgetrf does there. */
int pcbqs_gb300_lu_factor_c64(int64_t n, void *a, int32_t *ipiv, int block, int math, int32_t *singular,
                              void *stream);
/* Limit, in SM clocks, of the library's bounded device waits (a kernel waiting for its own copies, for other blocks
 * of a cooperative grid, or for its tensor-core products): a wait that runs out makes the call return
 * status 6 with the device context still usable. 0 restores the default (2^31, about a second).
 * Process-wide; read when a call launches its kernels. No counterpart in the reference (its CPU code has no device
 * waits); it lets a test make the waits run out without a fault. */
int pcbqs_gb300_set_wait_cycles(uint64_t cycles);
/* c -= a b for complex64 column-major device matrices (rows x k, k x cols, rows x cols; leading dimensions lda >= rows,
 * ldb >= k, ldc >= rows) on the tensor cores: this library's tcgen05 GEMM on BF16 parts of the FP32 values (terms 3:
 * h.h + h.m + m.h, about 2^-16 relative error per product; terms 6: also h.l + m.m + l.h, FP32's accuracy) with
 * FP32 accumulation, as one real GEMM of inner dimension terms * 2k. The trailing update of the blocked LU
 * (pcbqs_gb300_lu_factor_c64 math 2 and 3), exported so it can be checked on its own; the reference's counterpart is
 * LAPACK's cgemm inside cgetrf (MixedLU, src/pcbqs/kernels.py:150-151). Every wait inside the kernel gives up after
 * wait_cycles SM clocks (status 6). Takes its scratch from the library's memory pool; synchronizes
 * `stream`. */
int pcbqs_gb300_complex_update(int64_t rows, int64_t cols, int k, const void *a, int64_t lda, const void *b,
                               int64_t ldb, void *c, int64_t ldc, int terms, uint64_t wait_cycles, void *stream);
/* Dense FP32 Cholesky a = L L^T of the n x n column-major symmetric positive definite device matrix a (leading
 * dimension lda >= n, a multiple of 32 for the tensor-core GEMM forms; lower triangle read and overwritten by L;
 * the strict upper triangle is left with intermediate values), blocked like pcbqs_gb300_lu_factor_c64 (block 32 .. 4096, math 0: FP32 GEMMs, 1: BF16x9). *info
 * (host) = order of the first leading minor that is not positive definite, 0 if none. Synchronizes `stream`. No
 * counterpart in the reference: it is the factor of P behind pcbqs_gb300_dense_gmres's preconditioner, exported so
 * it can be checked on its own. */
int pcbqs_gb300_cholesky_f32(int64_t n, float *a, int64_t lda, int block, int math, int32_t *info, void *stream);
/* out = (complex64 factor)^-1 in for k complex128 columns (n, k) row-major, device arrays; the solve step of
 * MixedLU (src/pcbqs/kernels.py:160-181) without its refinement. method 0: what GMRES uses, this library's
 * streaming triangular sweeps (8 columns per pass over the factor) or its blocked solve whose off-diagonal products
 * run on the tcgen05 update (the factor read once for all columns), whichever the first call with this column
 * count timed faster; 2 / 3: the streaming / the blocked solve (validation); 1: cuSOLVER getrs on the same factor
 * (validation). Synchronizes `stream`. */
int pcbqs_gb300_peec_lu_solve(pcbqs_gb300_peec *op, int k, const double *in, double *out, int method,
                              void *stream);
/* Batched right-preconditioned restarted GMRES on k columns (b, x device; x holds the initial guess), relative
 * residual tol per column; iterations and residual (host, k) receive each column's Arnoldi steps and true
 * relative residual; precondition 0 none, 1 block-Jacobi, 2 the single-precision factor, 3 the graph
 * preconditioner (every column uses the factor or the graph preconditioner set up last).
 * Status 5 when a column did not converge. Replaces peec_iterative._gmres
 * (src/pcbqs/peec_iterative.py:100-112) and mqs_iterative._lockstep_gmres (src/pcbqs/mqs_iterative.py:109-170). */
int pcbqs_gb300_peec_gmres(pcbqs_gb300_peec *op, int k, const int32_t *sys, const double *b, double *x, double tol,
                           int maxiter, int restart, int precondition, int32_t *iterations, double *residual,
                           void *stream);
/* Y = M X for a dense symmetric real M (rows x rows, leading dimension ld, FP64) and complex128 X, Y (rows x k,
 * row-major), device arrays, in FP64 (the products of the loop/tree right-hand side and the charge correction,
 * src/pcbqs/peec_iterative.py:253-256, 331-341). Asynchronous on `stream`. */
int pcbqs_gb300_dense_apply(int64_t rows, int k, const double *M, int64_t ld, const double *X, double *Y,
                            void *stream);
/* The same product from the FP32 copy of M (the mixed solve's inner products), results in FP64. */
int pcbqs_gb300_dense_apply_single(int64_t rows, int k, const float *Mf, int64_t ld, const double *X, double *Y,
                                   void *stream);
/* The same product on the tcgen05 tensor cores: M's FP32 copy and X (rounded to FP32) split into BF16 parts, terms
 * 3 (relative error about 2^-16) or 6 (FP32's), one GEMM of inner dimension terms * rows against X's real and
 * imaginary columns side by side, FP32 accumulation. Packs M for this call only (the mixed solve packs L and P once
 * and reuses them) and synchronizes `stream`. Status 6 when a bounded wait (wait_cycles SM clocks) gave up. The
 * mixed solve's inner products take this path over 16 or more right-hand sides (pcbqs_gb300_peec_set_product). */
int pcbqs_gb300_dense_apply_tensor(int64_t rows, int k, const float *Mf, int64_t ld, const double *X, double *Y,
                                   int terms, uint64_t wait_cycles, void *stream);
/* The FP64 product (M FP64) to FP64's accuracy on the tcgen05 tensor cores: every row of M and every real column
 * of X is cut into `slices` (2..7) 8-bit integer slices under its own power-of-two scale (exact in BF16), the slice
 * products of each level summed exactly (FP32 over 256-long chunks, 32-bit integers across them) and the levels
 * carried into FP64. Error about 2^(-8 slices) of max_t |M[r,t]| sum_t |X[t,c]| (slices 6: 2^-48). Packs M for this
 * call only and synchronizes `stream`; status 6 when a bounded wait gave up. The operator's FP64 products take this
 * path over 4 or more right-hand sides after pcbqs_gb300_peec_set_fp64_product. */
int pcbqs_gb300_dense_apply_sliced(int64_t rows, int k, const double *M, int64_t ld, const double *X, double *Y,
                                   int slices, uint64_t wait_cycles, void *stream);
/* Single-precision copies of L and P (device, row strides ldlf/ldpf) for the inner products of the mixed solve,
 * and the conversion that makes them. */
int pcbqs_gb300_to_single(const double *in, float *out, int64_t count, void *stream);
int pcbqs_gb300_peec_single(pcbqs_gb300_peec *op, const float *Lf, int64_t ldlf, const float *Pf, const float *Pfim,
                            int64_t ldpf);
/* Mixed-precision solve: FP64 true residuals b - A x (the outer iterative refinement), each correction from an
 * inner right-preconditioned GMRES on the single-precision operator to inner_tol of the residual; until every
 * column's true relative residual <= tol or max_outer corrections. iterations: inner Arnoldi steps per column;
 * residual: final true relative residual; outer_steps: corrections made. The MixedLU scheme
 * (src/pcbqs/kernels.py:125-181) with a Krylov inner solve. */
int pcbqs_gb300_peec_solve_mixed(pcbqs_gb300_peec *op, int k, const int32_t *sys, const double *b, double *x,
                                 double tol, double inner_tol, int max_outer, int inner_maxiter, int restart,
                                 int precondition, int32_t *iterations, double *residual, int32_t *outer_steps,
                                 void *stream);
/* Partial inductance matrix of nv plated via segments (filaments along z): seg (device, nv x 5) rows (x, y, r, z0,
 * z1) in m, L (device, nv x nv, row stride ld) = scale [g(z1a - z0b) + g(z0a - z1b) - g(z1a - z1b) - g(z0a - z0b)],
 * g(u) = u asinh(u / s) - sqrt(u^2 + s^2), s the axis distance or, for coaxial segments and the self terms, the
 * larger radius; scale = mu0 / 4 pi. Ordered on `stream` (no synchronization). Replaces via_inductance and
 * filament_mutual (src/pcbqs/mqs.py:40-45, :140-153). */
int pcbqs_gb300_via_inductance(int64_t nv, const double *seg, double scale, double *L, int64_t ld, void *stream);
/* The learned block preconditioner (no counterpart in the reference, whose GMRES uses sparse surrogates; block
 * Jacobi is its fallback and the baseline it is trained against): out = y - sum_e g_e D_b^-1 A_bc y_c, y = D^-1 in,
 * over edges e = (b <- c) between blocks of bs unknowns, gains g_e = w2 . tanh(W1 phi_e + b1) + b2 from the edge
 * features phi_e (nfeat) with nhidden hidden units. params (device): W1 (nhidden x nfeat, row-major), b1, w2, b2.
 * Device arrays, FP64, complex interleaved; dinv (nblk, bs, bs) the inverted diagonal blocks (identity-padded),
 * E (nedge, bs, bs) the off-diagonal blocks (zero-padded), eptr (nblk + 1) / ecol (nedge) the edges grouped by
 * destination block. Ordered on `stream` (no synchronization) except learned_gmres. */
int pcbqs_gb300_learned_forward(int64_t nedge, int nfeat, int nhidden, const double *phi, const double *params,
                                double *hidden, double *gains, void *stream);
/* grad (device, nhidden * nfeat + 2 nhidden + 1) = dL/dparams for dgains = dL/dgains (deterministic sums). */
int pcbqs_gb300_learned_backward(int64_t nedge, int nfeat, int nhidden, const double *phi, const double *params,
                                 const double *hidden, const double *dgains, double *grad, void *stream);
/* out (n, k) = M^-1 in (gains null: block-Jacobi alone); corrections (nedge, bs, k), if not null, receives the
 * vectors u_e = D_b^-1 A_bc y_c (what the gains multiply). */
int pcbqs_gb300_learned_apply(int64_t n, int bs, int64_t nblk, const int64_t *eptr, const int32_t *ecol,
                              const double *dinv, const double *E, const double *gains, int k, const double *in,
                              double *out, double *corrections, void *stream);
/* dots[e] = sum over rows of block b and the k columns of Re(conj(S) u_e): with S = A^H r, the residual r's
 * derivative along each gain is -2 dots / |z|^2 for the loss |A M^-1 z - z|^2 / |z|^2. */
int pcbqs_gb300_learned_edge_dots(int64_t n, int bs, int64_t nblk, const int64_t *eptr, int k, const double *S,
                                  const double *corrections, double *dots, void *stream);
/* GMRES (this library's batched solver) on a dense complex row-major system A (n x n, row stride lda), k columns,
 * right-preconditioned by block-Jacobi (gains null) or the learned preconditioner; status 5 if a column did not
 * reach tol. iterations, residual: host arrays (k). Synchronizes `stream`. */
int pcbqs_gb300_learned_gmres(int64_t n, const double *A, int64_t lda, int k, const double *b, double *x, double tol,
                              int maxiter, int restart, int bs, int64_t nblk, const int64_t *eptr,
                              const int32_t *ecol, const double *dinv, const double *E, const double *gains,
                              int32_t *iterations, double *residual, void *stream);
/* A x = b for a dense symmetric A = A_re + j A_im (n x n, row stride lda; A_im nullable: real A) and k complex
 * columns by GMRES, preconditioned by the diagonal of A_re (precondition 0, as the reference) or by the
 * single-precision Cholesky factor of A_re (A_re positive definite; exact for a real A, a close preconditioner for
 * a lossy dielectric's complex potential matrix), its triangular solves by this library's streaming sweeps
 * (precondition 1: cooperative kernels, which need the device to themselves) or by cuBLAS (2: ordinary kernels, so
 * the solve may run while other work, such as a factorization on another stream, is in flight). Replaces peec_iterative.potential_solve
 * (src/pcbqs/peec_iterative.py:115-124), used for P^-1 B. */
int pcbqs_gb300_dense_gmres(int64_t n, const double *A, const double *Aim, int64_t lda, int k, const double *b,
                            double *x, double tol, int maxiter, int restart, int precondition, int32_t *iterations,
                            double *residual, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* PCBQS_GB300_H */
