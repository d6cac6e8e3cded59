/*
 * C ABI of the GB300 (sm_103a) engine for mom25d's per-frequency sweep path:
 * Green's-function tabulation, RWG impedance fill, dense complex LU factor +
 * solve, and port de-embedding to S-parameters.
 *
 * Every call returns an int status (M25_OK or an M25_ERR_* code); the text
 * of the last error of the calling thread is m25_last_error(). No C++
 * exception crosses this boundary. Array arguments are plain pointers with
 * sizes; "host" arrays are ordinary CPU memory, "device" arrays are CUDA
 * device pointers on the context's device. The engine works on its own
 * non-blocking stream (m25_ctx_stream): device inputs written on another
 * stream must be complete (synchronised, or ordered by an event) before the
 * call, and device outputs left on that stream (m25_assemble's Z) are
 * ordered for other streams by m25_ctx_synchronize or an event on it. Complex numbers are interleaved
 * (re, im) pairs of double (complex128) or float (complex64), row-major.
 *
 * Reference interfaces replaced (paths inside the mom25d project):
 *   m25_geometry_create  AssemblyGeometry.__init__  Engine/mom25d/solver.py:321-426
 *   m25_greens_create    GroundedSlabGreens          Engine/mom25d/greens.py:205-318
 *                        LayeredGreens               Engine/mom25d/layered.py:217-405
 *   m25_assemble         assemble                    Engine/mom25d/solver.py:429-524
 *                        _via_blocks                 Engine/mom25d/solver.py:527-566
 *   m25_dense_solve      _dense_solve                Engine/mom25d/solver.py:11-23
 *   m25_deembed          Solver.sweep de-embedding   Engine/mom25d/solver.py:1276-1325
 *                        (charges 1076-1091, line_voltage 1101-1125, PortModel 604-610,
 *                         fit_waves 618-670, _reciprocal_z0 1357-1427)
 *   m25_sweep_point      one iteration of Solver.sweep Engine/mom25d/solver.py:1273-1325
 *   m25_deembed_waves    SweepResult.waves           Engine/mom25d/solver.py:683, 1309
 *   m25_interp_*         FreqInterp                  Engine/mom25d/freqinterp.py:27-197
 *                        (and solve_currents' interpolated branch, solver.py:1012-1013)
 *   m25_mlp_*            (no counterpart: mom25d has no learned part) the
 *                        network of the learned Green's remainder, which
 *                        stands in for the Sommerfeld integrals of
 *                        Engine/mom25d/greens.py:157-173 / layered.py:360-372
 */
#ifndef M25_H
#define M25_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  M25_OK = 0,
  M25_ERR_VALUE = 1,   /* bad argument or model (mom25d raises ValueError) */
  M25_ERR_MEMORY = 2,  /* device memory exhausted (MemoryError) */
  M25_ERR_CUDA = 3,    /* CUDA runtime failure (RuntimeError) */
  M25_ERR_NUMERIC = 4  /* singular matrix, non-converged refinement (RuntimeError) */
};

/* Arithmetic of the path. M25_FP64: fp64 fill, fp64 LU. M25_MIXED: fp64 fill,
 * complex64 LU, fp64 GMRES refinement against the fp64 Z. M25_MIXED_FILL32:
 * fp32 fill (complex64 Z), complex64 LU, fp64 refinement against that Z. */
enum { M25_FP64 = 0, M25_MIXED = 1, M25_MIXED_FILL32 = 2 };
enum { M25_ON_HOST = 0, M25_ON_DEVICE = 1 };    /* where array arguments live */

typedef struct m25_ctx m25_ctx;
typedef struct m25_geom m25_geom;
typedef struct m25_greens m25_greens;

const char* m25_last_error(void);
int m25_version(void);

/* One context per host thread: a device, a CUDA stream, a workspace. */
int m25_ctx_create(int device, m25_ctx** out);
int m25_ctx_destroy(m25_ctx* ctx);
int m25_ctx_synchronize(m25_ctx* ctx);
/* free and total device memory of the context's device, in bytes */
int m25_ctx_mem_info(m25_ctx* ctx, uint64_t* free_bytes, uint64_t* total_bytes);
void* m25_ctx_stream(m25_ctx* ctx); /* the cudaStream_t every call of this context runs on */

/* Tuning knobs of this context's calls (no counterpart in mom25d; set per
 * point by mom25d_gb300/batch.py and Solver.sweep from the table autotune.py
 * measures), 0 keeping the process default: panel_cluster_min, the smallest
 * cluster (4, 8 or 16 CTAs) the LU panel runs on (default 4, or
 * $M25_PANEL_CLUSTER_MIN); wave_ctas, the CTA cap of the triangular solves
 * (default one per 64-row block, or $M25_WAVE_CTAS); tc_chunk, the steps of
 * 32 tf32 along K (12 MMAs each) the tensor-core update accumulates in TMEM
 * before adding into its fp32 registers (1..8; default 1, or $M25_TC_CHUNK:
 * longer chunks round the accumulation coarser); tc_tile_n, the N of the
 * tensor-core update's tiles in real columns (128 or 192; default 128 for
 * updates of at most 64 complex columns, 192 otherwise). */
int m25_ctx_set_tuning(m25_ctx* ctx, int32_t panel_cluster_min, int32_t wave_ctas, int32_t tc_chunk,
                       int32_t tc_tile_n);

/* Failure-path hook (no counterpart in mom25d, whose solve has no waits):
 * bound every ready-flag wait of this context's triangular solves to `polls`
 * polls (0 restores the default bound, about a second of polling). A solve
 * whose wait runs out returns M25_ERR_CUDA ("a wait of the triangular solve
 * ran out") after every block of the kernel has returned; the context stays
 * usable and its next solve starts with the error word cleared. Lets a test
 * make a wait run out on purpose without any fault. */
int m25_ctx_set_wait_limit(m25_ctx* ctx, int64_t polls);

/* Stage timers: CUDA events recorded on the context's stream around the
 * kernels of each stage (the verbose green / fill / solve timers of
 * Engine/mom25d/solver.py:1023-1026, per kernel class). Copies the
 * accumulated milliseconds and launch counts of the M25_STAGES stages to the
 * outputs (either may be NULL), then enable = 1 / 0 resets and switches the
 * timers on / off, enable = -1 only reads. Stages, in order: greens, fill,
 * gather, via, lu_panel, lu_pack (operand packing of the tensor-core update),
 * lu_swap_trsm (row interchanges + U12 solve), lu_gemm (trailing update),
 * trsv, refine, deembed. */
#define M25_STAGES 11
int m25_ctx_timing(m25_ctx* ctx, int enable, double* ms_out, long long* count_out);

/* ------------------------------------------------------------------ mesh */
typedef struct {
  int32_t nt, nb, nlev;       /* triangles, RWG bases, metal levels */
  const double* verts;        /* (nt,3,2) counter-clockwise vertices [m] */
  const int32_t* tri_basis;   /* (nt,3) basis of the edge opposite vertex i, -1 on a boundary */
  const double* tri_sign;     /* (nt,3) +1 (T+), -1 (T-), 0 */
  const double* edge_len;     /* (nb) */
  const int32_t* tri_layer;   /* (nt) level index */
  const double* level_z;      /* (nlev) level heights [m] */
  const int32_t* edge_tri;    /* (nb,2) T+, T- of each basis */
  const int32_t* edge_loc;    /* (nb,2) local index of the edge in T+, T- */
  int32_t nblocks;            /* test blocks: <= 32 Morton-ordered triangles of one level */
  const int32_t* block_tris;  /* (nblocks,32) triangle per slot, -1 empty */
  int32_t nv;                 /* via segments (unknowns nb .. nb+nv-1) */
  int32_t npad;               /* triangles attached to via ends */
  const int32_t* pad_tris;    /* (npad) */
  const int32_t* seg_pad_off; /* (nv+1) CSR offsets into seg_pad / seg_pad_w */
  const int32_t* seg_pad;     /* pad index per entry */
  const double* seg_pad_w;    /* +1/A_top or -1/A_bottom per entry */
  const int32_t* seg_end_lev; /* (nv,2) level of the top / bottom end charge, -1 none */
  const double* seg_span;     /* (nv,2) z bottom, z top [m] */
  const double* seg_xy;       /* (nv,2) via centre [m] */
  const double* seg_drill;    /* (nv) */
  double near_factor, far_factor; /* 3, 10 in mom25d */
} m25_mesh_desc;

/* Uploads the mesh, builds the frequency-independent fill data on the
 * device: quadrature points, near/mid/far classes per (test block, source
 * triangle), closed-form 1/R integrals of the near pairs. Host arrays. */
int m25_geometry_create(m25_ctx* ctx, const m25_mesh_desc* desc, m25_geom** out);
int m25_geometry_destroy(m25_geom* g);
/* out[0..3] = near, mid, far (test triangle, source triangle) pairs; bytes of near-pair data */
int m25_geometry_stats(m25_geom* g, int64_t* out4);

/* ---------------------------------------------------------- Green's tables */
typedef struct m25_mlp m25_mlp; /* learned remainder network, below */
typedef struct {
  double freq;
  int32_t nlayer;             /* dielectric layers, bottom to top (air above) */
  const double* layer_t;
  const double* layer_eps;
  const double* layer_tand;
  int32_t nlev;               /* metal levels of the mesh */
  const int32_t* lev_iface;   /* interface index 1..nlayer of each level */
  const double* lev_z;        /* height of each level [m] */
  int32_t single;             /* 1: one slab, metal on top (closed-form slab kernels) */
  double zs_ground_re, zs_ground_im; /* ground-plane surface impedance (0: PEC) */
  double stack_h;             /* total stack height [m] */
  int32_t nk_c, nk_r;         /* Sommerfeld path: lifted arc points, real-axis points */
  const double* kc;           /* (nk_c,2) complex points */
  const double* wc;           /* (nk_c,2) complex weights */
  const double* kr;           /* (nk_r) */
  const double* wr;           /* (nk_r) */
  int32_t nrho;
  const double* rho;          /* (nrho) tabulation radii, rho[0] = 0 */
  double kbig;                /* spectral sample for layered leading terms (15 / t_min) */
  /* Learned remainder (NULL: the Sommerfeld integral at every radius). The
   * network maps (2 log1p(rho/a) / log1p(rho_ref/a) - 1, 2 (f - fmin) /
   * (fmax - fmin) - 1) to the 2 NC scaled real and imaginary parts of the
   * remainder (NC = 3 nlev^2 columns [A, V, W] x level pairs, res = scale x
   * output). The Sommerfeld integral runs first at the knots (every radius
   * below sur_near, then every sur_stride-th radius and the last) and at one
   * validation radius in the middle of each gap between knots. A not-a-knot
   * spline of the residual (integral - network) through the knots, added to
   * the network, is judged at the validation radii: when its largest error
   * there is <= sur_tol x the largest |remainder|, the other radii take the
   * network plus a not-a-knot spline of the residual through all integrated
   * radii; else the Sommerfeld integral runs at them too. */
  const m25_mlp* surrogate;
  double sur_a, sur_rho_ref, sur_fmin, sur_fmax;
  const double* sur_scale;    /* (2 NC) */
  double sur_near;            /* [m] radii below it are always integrated */
  int32_t sur_stride;         /* 2 .. 64 */
  double sur_tol;
  int32_t top_pec;            /* 1: a PEC cover on the top layer (no level on it); 0: air above */
} m25_greens_desc;

int m25_greens_create(m25_ctx* ctx, const m25_greens_desc* desc, m25_greens** out);
int m25_greens_destroy(m25_greens* g);
/* Host copies: S (3,nlev,nlev,nrho) complex128 [S_A, S_V, S_W]; c (3,nlev,nlev)
 * complex128 leading coefficients; coef (nlev*nlev, nrho-1, 4, 3) complex128
 * not-a-knot cubic coefficients (highest power first). Any may be NULL. */
int m25_greens_tables(m25_greens* g, double* S, double* c, double* coef);
/* The Sommerfeld remainder the tables were built from: res (nrho, NC)
 * complex128 (surrogate tables: the corrected network values);
 * info[0] = 1 if the learned remainder was used, info[1] = the judge's
 * relative error (0 without a surrogate), info[2] = the number of radii the
 * Sommerfeld integral ran at. Either may be NULL. */
int m25_greens_remainder(m25_greens* g, double* res, double* info);

/* ------------------------------------------------ learned remainder (MLP) */
/* A tanh MLP in fp32 on the device: n_in (<= 4) inputs, n_layers (1..4)
 * hidden layers of width hidden (= 64), n_out (<= 64) linear outputs.
 * Parameters (one float array, layer by layer: W (out, in) row-major, then b)
 * start Glorot-uniform from seed, biases zero. */
int m25_mlp_create(m25_ctx* ctx, int32_t n_in, int32_t hidden, int32_t n_layers, int32_t n_out, uint64_t seed,
                   m25_mlp** out);
int m25_mlp_destroy(m25_mlp* m);
/* *count = parameter count; get / set (host float32, count) may be NULL */
int m25_mlp_params(m25_mlp* m, int64_t* count, float* get, const float* set);
/* loss = mean over samples and outputs of (f(X) - Y)^2 and its gradient
 * (host float32: X (n, n_in), Y (n, n_out), grad (count)) */
int m25_mlp_loss_grad(m25_mlp* m, int32_t n, const float* X, const float* Y, double* loss, float* grad);
/* Adam (0.9, 0.999, 1e-8) on minibatches of `batch` rows drawn from (X, Y)
 * by a counter-based hash of seed, learning rate cosine-decayed from lr to
 * lr_min over `steps`; loss_out = the loss over all n samples afterwards */
int m25_mlp_train(m25_mlp* m, int32_t n, const float* X, const float* Y, int32_t steps, int32_t batch, double lr,
                  double lr_min, uint64_t seed, double* loss_out);
int m25_mlp_forward(m25_mlp* m, int32_t n, const float* X, float* Y);

/* ----------------------------------------------------------------- fill */
/* Z (n x n, n = nb + nv) of the MPIE Galerkin fill, symmetrised. precision
 * M25_FP64 and M25_MIXED write complex128 (fp64 arithmetic), M25_MIXED_FILL32
 * complex64 (fp32 arithmetic). Z is host or device memory (where); ldz its
 * row stride in elements. */
int m25_assemble(m25_ctx* ctx, m25_geom* geom, m25_greens* gr, double zs_re, double zs_im,
                 double zsv_re, double zsv_im, int precision, void* Z, int64_t ldz, int where);

/* ---------------------------------------------------------------- solve */
/* Z X = B for an n x n complex128 Z (overwritten by its LU factors when on
 * the device, as mom25d's _dense_solve overwrites Z) and nrhs right-hand
 * sides B (n x nrhs complex128, row-major). precision M25_FP64: LU with
 * partial pivoting in fp64 (Z complex128); M25_MIXED: Z complex128, LU of its
 * complex64 copy, fp64 GMRES refinement against Z until the normwise backward
 * error |r| / (|Z| |x| + |b|) <= tol within max_iter GMRES steps;
 * M25_MIXED_FILL32: the same with a complex64 Z. info[0] = GMRES steps,
 * info[1] = 0 or the first zero pivot (1-based). */
int m25_dense_solve(m25_ctx* ctx, int32_t n, int32_t nrhs, int precision, void* Z, const void* B, void* X,
                    int where, double tol, int32_t max_iter, int32_t* info);

/* In-place LU factorisation with partial pivoting of an n x n row-major matrix
 * (scipy.linalg.lu_factor, used by _dense_solve, Engine/mom25d/solver.py:23):
 * precision M25_FP64 factors complex128, M25_MIXED complex64 (trailing
 * updates on the tensor cores unless flags & M25_LU_NO_TENSOR_CORES). On
 * return A holds L (unit lower, strictly below the diagonal) and U, ipiv the
 * 0-based row interchanges (row i swapped with ipiv[i], in order). A and ipiv
 * are host or device memory (where). info = first zero pivot (1-based) or 0. */
#define M25_LU_NO_TENSOR_CORES 1
int m25_lu_factor(m25_ctx* ctx, int32_t n, int precision, void* A, int64_t lda, int32_t* ipiv, int where,
                  int32_t flags, int32_t* info);

/* Allocation-free dense solve (no counterpart in mom25d). For callers that
 * must not allocate device memory themselves or through this library:
 * applications whose device memory belongs to another allocator (a
 * framework's caching allocator, a fixed arena sized at start-up) and that
 * cannot let a library call cudaMalloc / cudaFree in the middle of their
 * work, since those calls synchronise the device and fail once the arena
 * holds the memory. The same computation as m25_dense_solve with M25_FP64
 * (complex128 LU with partial pivoting, then the two triangular solves), on
 * caller-owned device memory only: Z (n x n complex128, row-major,
 * overwritten by its LU factors), B (n x nrhs complex128, read only), X
 * (n x nrhs complex128, the solution), ipiv (n int32, the 0-based pivot rows),
 * on `stream` (a cudaStream_t; NULL = the legacy default stream). The
 * library's own scratch is one static device array of
 * M25_NOALLOC_SCRATCH_BYTES that every GPU loading the library keeps until
 * the process exits; it limits n to M25_NOALLOC_MAX_N (larger n is rejected
 * with M25_ERR_VALUE) and the device to at most 192 SMs. The first call on a
 * device looks up the array's device address (cudaGetSymbolAddress, with that
 * device current). All calls share the one array: calls that overlap on the
 * GPU (other threads, other streams) race and must be serialised by the
 * caller. info[0] = 0, info[1] = the first zero pivot (1-based) or 0. Every
 * call blocks the calling thread until `stream` has finished the solve (the
 * factorisation reads its pivot flags and the triangular solves their error
 * word on the host), so no call can be captured into a CUDA graph. */
#define M25_NOALLOC_MAX_N 24576
#define M25_NOALLOC_SCRATCH_BYTES (512 * 1024)
int m25_dense_solve_noalloc(int32_t n, int32_t nrhs, void* Z, const void* B, void* X, int32_t* ipiv, void* stream,
                            int32_t* info);

/* ----------------------------------------------------------- de-embedding */
typedef struct {
  int32_t nport;               /* feed ports P */
  int32_t ngroup;              /* ports sharing a line (same width, level): one wave fit each */
  const int32_t* group_of;     /* (P) group index */
  const int32_t* port_level;   /* (P) mesh level of each feed */
  const int32_t* ns;           /* (P) fit-window cuts per port */
  const double* s;             /* concatenated cut positions [m] */
  const int32_t* cut_off;      /* (sum ns + 1) CSR over cut edges */
  const int32_t* cut_edge;     /* RWG index per entry */
  const double* cut_w;         /* sign * edge length per entry */
  const int32_t* nvpt;         /* (P) voltage points per port (ns * 8) */
  const double* vpts;          /* concatenated (x, y) voltage points */
  const double* beta0;         /* (ngroup) Kirschning-Jansen initial phase constant */
  int32_t lossless;            /* 1: bounded Brent on beta; 0: Nelder-Mead on gamma */
  const double* bounds;        /* (ngroup,2) beta search bounds (lossless) */
  double v_weight;             /* voltage residual weight (1) */
  const double* excitation;    /* (nport, n) delta-gap excitation vectors (PortModel.excitation) */
} m25_port_desc;

typedef struct m25_ports m25_ports;
int m25_ports_create(m25_ctx* ctx, m25_geom* geom, const m25_port_desc* desc, m25_ports** out);
int m25_ports_destroy(m25_ports* p);

/* From the solution x (n x P complex128, device or host per where) at one
 * frequency: S (P,P) referenced to the extracted line impedances, z0 (P),
 * gamma (P), z0_line (P), fit residual (P), all host complex128 / float64.
 * beta0 overrides the per-group initial guess (NULL: from the port desc). */
int m25_deembed(m25_ctx* ctx, m25_geom* geom, m25_greens* gr, m25_ports* ports, const void* x, int where,
                const double* beta0, double* S, double* z0, double* gamma, double* z0_line, double* resid);

/* Internal ports (Layout.add_gap_port / add_via_port, Engine/mom25d/
 * solver.py:1029-1034, 1305-1318): the solutions handed to m25_deembed carry
 * nexc columns, the P feed excitations then one per internal port. Every
 * feed's wave fit then takes its currents and voltages under all nexc
 * excitations (P <= nexc <= 8, at most 16 (port, excitation) datasets per
 * port group), m25_deembed returns gamma, z0_line and the residual but not
 * S, and m25_deembed_coefs gives the fitted amplitudes A and B (P x nexc
 * complex128, [port][excitation]) from which the caller assembles S with the
 * internal ports' rows. nexc = P restores the feed-only de-embedding. */
int m25_ports_set_excitations(m25_ports* ports, int32_t nexc);
int m25_deembed_coefs(m25_ports* ports, double* A, double* B);

/* Per port group, the iterations of the last de-embedding's wave fit
 * (Nelder-Mead, or for a lossless stack the bounded Brent search over beta);
 * a lossless fit whose beta ended within 1e-3 |beta0| of its search bound
 * reports minus its iterations: mom25d warns that gamma, Z0 and S are
 * unreliable there (fit_waves, Engine/mom25d/solver.py:654-662). */
int m25_deembed_fit_info(m25_ports* ports, int32_t* iters);

/* One frequency point of Solver.sweep (Engine/mom25d/solver.py:1273-1325) with
 * every intermediate on the device: fill (precision), solve of the port
 * excitations, de-embedding. x_out (n, P) complex128 host copy of the
 * currents or NULL; S, z0, gamma, z0_line, resid as m25_deembed; info[0]
 * refinement steps, info[1] zero pivot. When the mixed refinement does not
 * reach tol (the complex64 LU too inaccurate at that frequency) the point is
 * recomputed on the fp64 path and info[0] = -1. */
int m25_sweep_point(m25_ctx* ctx, m25_geom* geom, m25_greens* gr, m25_ports* ports, double zs_re, double zs_im,
                    double zsv_re, double zsv_im, int precision, const double* beta0, double tol, int32_t max_iter,
                    double* x_out, double* S, double* z0, double* gamma, double* z0_line, double* resid,
                    int32_t* info);

/* ---- Frequency interpolation of Z (FreqInterp, Engine/mom25d/freqinterp.py:27-197).
 * Anchor matrices W = j w Z exp(+j k_e R) are kept on the device in nslots
 * slots (complex128, or complex64 when single != 0); at another frequency
 * Z = (sum_a L[a] W[slot[a]]) exp(-j k_e R) / (j w). R is the distance of the
 * basis centres pos (n x 3, host float64: RWG edge midpoints on their level,
 * via segments at mid-span), 0 between two via unknowns (rows and columns
 * >= nb); k_e = k_ratio w / c0. Z is n x n complex128, rows ldz apart, on the
 * device or the host per where. */
typedef struct m25_interp m25_interp;
int m25_interp_create(m25_ctx* ctx, int32_t n, int32_t nb, const double* pos, int32_t nslots, int32_t single,
                      m25_interp** out);
int m25_interp_destroy(m25_interp* ip);
/* slot <- W of the given Z at freq (FreqInterp._anchor, freqinterp.py:107-122) */
int m25_interp_store(m25_interp* ip, int32_t slot, const void* Z, int64_t ldz, int where, double freq, double ke);
/* Z <- the interpolation at freq from nuse <= 8 slots with weights L
 * (FreqInterp.impedance, freqinterp.py:145-165) */
int m25_interp_eval(m25_interp* ip, int32_t nuse, const int32_t* slots, const double* L, double freq, double ke,
                    void* Z, int64_t ldz, int where);
/* Fill Z at the anchor frequency of gr (precision as m25_assemble; M25_MIXED
 * and M25_FP64 give complex128) and store it in slot. */
int m25_interp_anchor(m25_ctx* ctx, m25_geom* geom, m25_greens* gr, m25_interp* ip, int32_t slot, double zs_re,
                      double zs_im, double zsv_re, double zsv_im, int precision, double ke);
/* One frequency point as m25_sweep_point with the interpolated Z in place of
 * the fill (Solver.sweep with a FreqInterp, solver.py:1273-1325 and
 * solve_currents 1012-1013): solve (precision M25_FP64 or M25_MIXED), then
 * de-embedding with the tables of gr. A mixed solve that does not reach tol
 * is redone in fp64 on the same interpolated Z (info[0] = -1). ctx may be any
 * context of the anchors' device: the anchors are read-only here, and the
 * fills that wrote them must be complete (m25_ctx_synchronize on theirs). */
int m25_interp_point(m25_ctx* ctx, m25_geom* geom, m25_greens* gr, m25_ports* ports, m25_interp* ip, int32_t nuse,
                     const int32_t* slots, const double* L, double ke, int precision, const double* beta0, double tol,
                     int32_t max_iter, double* x_out, double* S, double* z0, double* gamma, double* z0_line,
                     double* resid, int32_t* info);

/* Incident current-wave amplitudes A (P, P) complex128 host, row = port,
 * column = excitation, of the last de-embedding on these ports (m25_deembed,
 * m25_sweep_point, m25_interp_point): SweepResult.waves, solver.py:683,
 * 1309-1312 (S = D (-B A^-1) D^-1). */
int m25_deembed_waves(m25_ports* ports, double* A);

/* Diagnostics of the last m25_deembed: phi (sum nvpt, P) complex128 line
 * voltages, q (nt, P) complex128 triangle charges, I and V (sum ns, P)
 * complex128 cut currents / voltages. NULL skips an output. */
int m25_deembed_debug(m25_ctx* ctx, m25_ports* ports, double* phi, double* q, double* I, double* V);

/* ---- Compressed operator (H-matrix) and its GMRES solve (Engine/mom25d/
 * hmatrix.py:145-606, HOperator: assemble, matvec, solve). The host builds
 * the cluster tree and the block partition; every range below is in tree
 * order (position k holds RWG basis perm[k]; the via unknowns follow at nb).
 * near: leaf pairs (a0, am, b0, bn), both orders; far: admissible pairs
 * (r0, m, c0, n), each unordered pair once, far_cen 1 for the centroid rule;
 * ent: per leaf (CSR ent_off) the items of its rows (type 0 near pair id,
 * 1 far block whose rows hold the leaf, 2 far block whose columns hold it;
 * id; the leaf's offset inside the block's rows / columns; 0); keys: the
 * near field's (test block x nt + source triangle) pairs, sorted; pblk: the
 * test blocks holding via pad triangles; preconditioner blocks (restricted
 * additive Schwarz): per block its unknowns (RWG positions of whole leaves,
 * then vias; at most 1024), which of them it writes, and per (row leaf,
 * column leaf) pair of its leaves the source of that sub-block (a near pair
 * id, or nnear + 2 f for far block f as rows, + 1 as its transpose) with the
 * sub-block's local row and column. rules: per basis 40 values of the far-field rules
 * (3-point points, w cA (r - a), w cV; centroids, A cA (c - a), A cV). */
typedef struct m25_hmat m25_hmat;
typedef struct {
  int32_t nb, nv;
  const int32_t* perm;
  const double* rules;
  const int32_t* lev;
  int32_t nleaf;
  const int32_t* leaf_lo;     /* (nleaf + 1) */
  int32_t nnear;
  const int32_t* near;        /* (nnear, 4) */
  int32_t nfar;
  const int32_t* far;         /* (nfar, 4) */
  const int32_t* far_cen;     /* (nfar) */
  const int64_t* ent_off;     /* (nleaf + 1) */
  const int32_t* ent;         /* (ent_off[nleaf], 4) */
  int64_t nkeys;
  const int64_t* keys;
  int32_t npblk;
  const int32_t* pblk;
  int32_t npc;
  const int64_t* pc_off;      /* (npc + 1) CSR of the blocks' unknowns */
  const int32_t* pc_gidx;     /* vector index of each block unknown (tree position, or nb + via) */
  const int8_t* pc_own;       /* 1: the block writes this unknown (each unknown owned once) */
  const int64_t* pc_item_off; /* (npc + 1) */
  const int32_t* pc_items;    /* (pc_item_off[npc], 5): source, row leaf, column leaf, local row, local column */
  double tol;                 /* ACA tolerance (1e-4) */
  int32_t kcap;               /* most ACA terms stored per block */
} m25_hmat_desc;
int m25_hmat_create(m25_ctx* ctx, m25_geom* geom, const m25_hmat_desc* desc, m25_hmat** out);
int m25_hmat_destroy(m25_hmat* h);
/* Near field (exact entries of the dense fill), far blocks (ACA, or stored
 * as they are), via blocks and the preconditioner at the tables' frequency.
 * stats (8, or NULL): near entries, low-rank blocks, far blocks stored as they
 * are, far entries held, largest rank, sum of ranks, blocks not low rank,
 * near-field triangle pairs. */
int m25_hmat_assemble(m25_hmat* h, m25_greens* gr, double zs_re, double zs_im, double zsv_re, double zsv_im,
                      int64_t* stats);
/* y = Z x with the compressed operator; x, y host complex128 (n). */
int m25_hmat_matvec(m25_hmat* h, const double* x, double* y);
/* X = Z^-1 B by flexible restarted GMRES on the symmetrically scaled system
 * W Z W (W = |Z_ii|^-1/2), column by column; B, X host complex128 (n, nrhs)
 * row-major; iters and resid (the scaled system's true relative residual)
 * per column. A column that does not reach rtol returns M25_OK with its
 * residual (the caller accepts or raises, as mom25d does). */
int m25_hmat_solve(m25_hmat* h, int32_t nrhs, const double* B, double* X, double rtol, int32_t restart,
                   int32_t maxiter, int32_t* iters, double* resid);

#ifdef __cplusplus
}
#endif

#endif /* M25_H */
