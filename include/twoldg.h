/*
 * twoldg.h -- C ABI of libtwoldg, the GB300 (sm_103a) implementation of the
 * OLDG field right-hand side and RK4 time step of TreeWaveOLDG.jl.
 *
 * Plain C: no C++ or torch types in any signature, so Julia `ccall`, Python
 * ctypes or any FFI can bind it. Every call returns an int status (0 = ok,
 * else one of TWOLDG_E*); twoldg_last_error() gives the text of the most
 * recent failure on the calling thread.
 *
 * Ownership: the caller owns the state vectors (device pointers in the
 * reference's state layout (N^D, 2, nblocks), column-major, u then v per
 * block, src/stepping.jl:24-25), so `pointer(::CuArray)` passes straight
 * through. The library owns its ghost/face buffers, stage scratch, tables
 * and one CUDA stream per problem; calls on one problem are not
 * thread-safe. All calls are asynchronous on the problem's stream except
 * those that return host scalars (energy, norm) and twoldg_synchronize.
 */
#ifndef TWOLDG_H
#define TWOLDG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TWOLDG_OK 0
#define TWOLDG_EINVAL 1     /* bad descriptor or argument (host-checked) */
#define TWOLDG_ECUDA 2      /* a CUDA call failed */
#define TWOLDG_ENOMEM 3     /* device allocation failed */
#define TWOLDG_EUNSUP 4     /* valid but not supported by this build (e.g. order, block size) */

#define TWOLDG_F64 0        /* plain FP64: the drop-in */
#define TWOLDG_F32 1        /* FP32 fields and stencil */
#define TWOLDG_F32C 2       /* FP32 fields, compensated (two-sum) RK4 accumulation */

/*
 * A forest of blocks in the form TreeAMR's Forest holds it (a brick of
 * roots[d] root blocks per dimension, each leaf a block at `level` whose
 * integer corner `corner[b*dim + d]` counts blocks of that level from the
 * domain's low corner), with the element layout of the reference's
 * element-centered field sets: N = elems * (order + 1) nodes per block and
 * dimension, `elems` even (src/layout.jl:31-47). Faces are periodic,
 * reflecting (solid wall: u, v even, d_d u odd; src/evolution.jl:1025-1027)
 * per dimension; a forest may be refined with 2:1 face balance, and its
 * coarse-fine faces get the element-local prolongation / restriction
 * ghosts. Blocks are numbered in the caller's order, which is the state
 * layout's block order.
 */
#define TWOLDG_FACE_BRICK (-2)  /* face_nb: a face between two blocks of a refined brick patch */

typedef struct twoldg_desc {
    int32_t dim;             /* D = 1, 2 or 3 */
    int32_t order;           /* P, 1 to 8 (TWOLDG_EUNSUP beyond) */
    int32_t elems;           /* E, even */
    int32_t precision;       /* TWOLDG_F64 / TWOLDG_F32 / TWOLDG_F32C */
    int32_t truncate;        /* 1: v held at degree P-1 (the paper's scheme) */
    int32_t nblocks;
    int32_t roots[3];
    int32_t periodic[3];
    int32_t reflecting[3];
    double lo[3];
    double hi[3];
    const int32_t* level;    /* nblocks */
    const int64_t* corner;   /* nblocks * dim */
    /* Optional diagonal metric (a geometry such as the polar annulus,
     * src/evolution.jl:513-708): NULL for the flat problem. coef holds, per
     * block, the node values of sqrt(g), A_1 .. A_D with A_d = sqrt(g) g^dd,
     * laid out (N^D, 1 + D, nblocks) column-major like the state; the gradient
     * then holds the flux A_d D_d u and the Laplacian divides by sqrt(g).
     * trunc_modes / trunc_duals hold the truncation's rank-one pair of every
     * element line, orthogonal in the sqrt(g)-factor-weighted inner product
     * (MetricTruncation, src/evolution.jl:556-622): for each dimension d, block
     * b and element index e along d, P+1 values, laid out (P+1, E, nblocks, D)
     * column-major. Both are rounded once to the field type. A problem with a
     * metric takes no coarse-fine faces and no batching. */
    const double* coef;
    const double* trunc_modes;
    const double* trunc_duals;
    /* The metric's kind: 0 flat (coef NULL), 1 diagonal (coef: sqrt(g), A_d),
     * 2 full (a geometry whose glues may swap axes, such as the seven-patch
     * ball, src/evolution.jl:112-220, D = 3 only): coef then holds sqrt(g) and
     * the area vectors S[d][i] = sqrt(g) d xi^d / d x^i at 1 + D d + i,
     * (N^D, 1 + D^2, nblocks), and the gradient crosses faces as Cartesian
     * components. */
    int32_t metric;
    /* An explicit face table for a forest of glued patches (NULL: the brick
     * of roots above): face_nb[b*2D + f] is the block across face f of block
     * b, or -1 for a face on the domain's boundary, which takes the Dirichlet
     * data below; face_code[b*2D + f] = (the neighbour's face) | (o << 4),
     * where o maps this face's tangential point (a, b) to the neighbour's:
     * bit 0 swaps a and b, bit 1 then reverses the first, bit 2 the second.
     * One patch may be a refined brick (the ball's affine cube, refined as
     * src/geometry.jl:494-553 refines it): the faces between its blocks are
     * TWOLDG_FACE_BRICK, and those blocks give their level and their corner
     * (in blocks of that level) in a brick of roots[d] root blocks, whose
     * faces the library resolves by level and corner, coarse-fine faces
     * included (the element-local I and R of the flat problem). Explicit
     * faces join blocks of one level. */
    const int32_t* face_nb;
    const int32_t* face_code;
    /* The full metric's truncation (ElementTruncation, src/evolution.jl:723-899):
     * elem_slot[b] = 0 takes the element's tensor projector (a block of an
     * affine patch), s >= 1 the tables s - 1 of elem_w ((P+1)^D, E^D, elem_ntab:
     * quadrature weights times sqrt(g)) and elem_chol (P^D, P^D, E^D, elem_ntab:
     * the upper Cholesky factor U of the Gram matrix, G = U^T U), column-major. */
    const int32_t* elem_slot;
    const double* elem_w;
    const double* elem_chol;
    int32_t elem_ntab;
    /* Dirichlet data on boundary faces: the plane wave u = sin(k . x - |k| t +
     * phi) (src/sevenpatch.jl:9-36); bnd_x holds, for every face slot b*2D + f,
     * the physical positions of its face nodes, (N^(D-1), 3) per slot (only the
     * boundary faces' are read). */
    double wave_k[3];
    double wave_phi;
    const double* bnd_x;
    /* The boundary faces' condition: 0 the Dirichlet plane wave above; 1 the
     * radiative, maximally dissipative condition n . grad u = -(kappa du/dt +
     * inv_r u) (RadiativeBoundary, src/evolution.jl:1129-1260): u's ghost is
     * the face node's own u, and the gradient's ghost makes the flux through
     * the face F* = -sigma |S[d]| (kappa v + inv_r u), sigma = -1 on a low
     * face and +1 on a high one. kappa >= 0; inv_r = 1/R, or 0 without the u/R
     * term. The energy then carries the boundary's own term,
     * 1/2 inv_r sum w |S[d]| u^2 over the boundary faces' nodes; 2 Dirichlet
     * data of any form, whose values the caller supplies at the stage times
     * (twoldg_set_boundary_values). */
    int32_t boundary;
    double kappa;
    double inv_r;
    /* The factored truncation (FactoredTruncation, src/evolution.jl:759-899)
     * of blocks whose sqrt(g) is a radial factor along one dimension times an
     * angular factor across it (the thirteen-patch ball's outer shells), NULL
     * when there are none: fac_slot[b] = 0 for any other block and f + 1 for the
     * factored block f; fac_radial[f] its radial dimension (0-based);
     * fac_rmodes / fac_rduals (P+1, E, nfac) the rank-one pair along it per
     * element index; fac_aslot[f] its angular tables among fac_ntab: fac_aw
     * ((P+1)^2, E^2, fac_ntab), the in-plane quadrature weights times the
     * angular factor, and fac_achol (P^2, P^2, E^2, fac_ntab), the upper
     * Cholesky factor of the in-plane Gram matrix; in-plane nodes, elements
     * and modes run over the two dimensions across the radial one in
     * increasing order, the first fastest. Such a block has elem_slot 0. */
    const int32_t* fac_slot;
    const int32_t* fac_radial;
    const double* fac_rmodes;
    const double* fac_rduals;
    const int32_t* fac_aslot;
    const double* fac_aw;
    const double* fac_achol;
    int32_t fac_ntab;
} twoldg_desc;

typedef struct twoldg_problem twoldg_problem;

const char* twoldg_last_error(void);
const char* twoldg_version(void);

/* Element tables of order P rounded once to float64 (precision 0) or float32
 * (precision 1), for the host side's node positions and for tests:
 * src/element.jl:129-170 (Element(T, P)). Arrays are row-major; `out` must
 * hold table_size(P) words of the requested type. Sizes per order P:
 * nodes, weights, offsets: P+1; stencil (P+1)(P+3); truncate (P+1)^2;
 * topmode, topdual: P+1; duals (P+1)^2; prolong 2(P+1)^2; restrict 2(P+1)^2. */
int twoldg_element_tables(int32_t order, int32_t precision, const char* name, void* out);

/* WaveProblem(forest, el; truncate) -- src/evolution.jl:1043-1108.
 * Builds the neighbour and coarse-fine face tables, uploads the tables and
 * allocates the scratch. */
int twoldg_problem_create(const twoldg_desc* desc, twoldg_problem** out);
int twoldg_problem_destroy(twoldg_problem* p);

/* Words of the state vector: N^D * 2 * nblocks. */
int twoldg_state_words(const twoldg_problem* p, int64_t* words);
/* Smallest block spacing (the finest level's) -- minimum_spacing(forest). */
int twoldg_min_spacing(const twoldg_problem* p, double* h);

/* wave_rhs!(du, u, p, t) -- src/evolution.jl:1367-1371: du = (v, sum_d D_d D_d u).
 * Does not truncate, never writes u. */
int twoldg_rhs(twoldg_problem* p, void* du, const void* u, double t);

/* truncate_state!(u, p) -- src/evolution.jl:1383-1395: v <- (Pi x ... x Pi) v
 * per element, in place; no-op when the problem does not truncate. */
int twoldg_truncate(twoldg_problem* p, void* u);

/* `nsteps` classic RK4 steps of size dt from time t, in place on u, with the
 * truncation as stage and step limiter -- wave_integrator + solve!
 * (src/stepping.jl:72-78, src/evolution.jl:1408-1430). The steps run from
 * CUDA graphs of up to 16 steps (a call's remainder in a graph of its own),
 * captured on first use for a (state pointer, step count) pair; the six most
 * recently used graphs are kept (a caller may alternate state buffers), and
 * a new dt changes only the coefficients the graphs read.
 * For TWOLDG_F32C the compensation words persist between calls on the same
 * u and are cleared when u changes or by twoldg_reset_compensation. */
int twoldg_rk4_step(twoldg_problem* p, void* u, double t, double dt, int32_t nsteps);
int twoldg_reset_compensation(twoldg_problem* p);

/* wave_energy(p, u) -- src/evolution.jl:1472-1489: 1/2 sum w (v^2 + sum_d (D_d u)^2),
 * FP64 accumulation, deterministic order. Synchronous. */
int twoldg_energy(twoldg_problem* p, const void* u, double t, double* energy);

/* quadrature_norm(fs, el, u; p, vars) -- src/layout.jl:223-235, of u - ref
 * when ref is not NULL. p >= 1, or p = 0 for the largest |value| (p = Inf).
 * vars_mask bit 0 = u, bit 1 = v. FP64 accumulation. Synchronous. */
int twoldg_norm(twoldg_problem* p, const void* u, const void* ref, int32_t pnorm, int32_t vars_mask,
                double* out);

/* modal_indicator(fs, el; mode, var) -- src/refinement.jl:147-155 (mode_kernel!
 * :56-77): tau[e1..eD, b] = max over lines and m = 1..mode of
 * (|c_m| (2m-1)!!/A)^(mode/m) / (2 mode - 1)!!, A the global peak |var|.
 * var is 1 (u) or 2 (v); tau_dev holds E^D * nblocks words of the field type. */
int twoldg_modal_indicator(twoldg_problem* p, const void* u, int32_t var, int32_t mode, void* tau_dev);
/* mode_amplitude(fs, el; mode, var) -- src/refinement.jl:169-175. */
int twoldg_mode_amplitude(twoldg_problem* p, const void* u, int32_t var, int32_t mode, void* tau_dev);

/* Diagnostics (no reference counterpart): runs one RK4 step of size dt on u
 * without the graph, with CUDA events between the four stages, and returns
 * each stage's duration in milliseconds (stage_ms[4]). Synchronous. */
int twoldg_profile_step(twoldg_problem* p, void* u, double dt, float* stage_ms);
/* Dirichlet data of any form, data(x, t) -> (u, grad u), on the boundary
 * faces of a full-metric problem with boundary = 2: the reference's
 * DirichletValues{:u} and {:grad} through boundary_by_coordinates
 * (src/evolution.jl:1110-1127, 1303-1314), which evaluate a Julia function at
 * every ghost; here the caller evaluates it (with a kernel of its own, as the
 * reference's launch_points! runs a closure) into a device table the library
 * reads. twoldg_boundary_faces lists the boundary faces' slots b*6 + f in the
 * order the table uses (slots NULL: only *n, their number); their nodes'
 * positions are the descriptor's bnd_x of those slots.
 * twoldg_set_boundary_values hands the table over: `values` (device, FP64)
 * holds nlevels time levels t0 + k dt/2, each level nbf faces, each face u at
 * its N^2 face nodes and then the three Cartesian components of grad u, N^2
 * each: values[((k * nbf + j) * 4 + c) * N^2 + t]. The library keeps the
 * pointer: the table must stay on the device, unchanged, until the work that
 * reads it is done. A call at time t reads level (t - t0) / (dt/2); rk4_step
 * from t of nsteps steps of size dt reads the 2 nsteps + 1 levels from t on,
 * and needs the table's dt; twoldg_rhs and twoldg_energy at t read t's level.
 * Each such call is refused (TWOLDG_EINVAL) when the table does not hold its
 * times. Asynchronous on the problem's stream. */
int twoldg_boundary_faces(twoldg_problem* p, int32_t* slots, int32_t* n);
int twoldg_set_boundary_values(twoldg_problem* p, const double* values, int32_t nlevels, double t0, double dt);

/* Diagnostics (no reference counterpart): times, with CUDA events on the
 * problem's stream, one launch each of the kernels around the stage kernel,
 * on the state u (not changed): ms[0] the face export (export_faces_kernel),
 * ms[1] the coarse-fine ghosts (cf_ghost_kernel; 0 without coarse-fine
 * faces), ms[2] the energy's reduction (energy_kernel, after that export),
 * ms[3] the norm of u - u (norm_kernel, p = 2, both variables), ms[4] the
 * indicator's peak (maxabs_kernel, u), ms[5] the modal indicator up to mode
 * max(P - 1, 1) (mode_kernel, u), ms[6] the truncation of a copy of u
 * (truncate_kernel). n must be at least 7. Flat and diagonal problems only.
 * Synchronous. */
int twoldg_profile_kernels(twoldg_problem* p, const void* u, float* ms, int32_t n);
/* The extraction's gather (sphere_values / plane_values, src/extraction.jl:
 * 216-245): out[j] = sum_q weights[q + nper j] * u[index[q + nper j] + (var-1)
 * N^D] for j < npoints, the element polynomials of variable var (1: u, 2: v)
 * at located points. index (int64, positions in the state vector for
 * variable 1), weights and out are device arrays, weights and out of the
 * problem's field type; the host builds the stencils (the points' elements
 * and Lagrange weights). Asynchronous on the problem's stream. */
int twoldg_gather(twoldg_problem* p, const void* u, int32_t var, int64_t npoints, int32_t nper,
                  const int64_t* index, const void* weights, void* out);

/* The regrid transfer (TreeAMR's element-set regrid, which the reference's
 * regrid! / adaptive_blast run on the host: src/blast.jl, CODE.md "Adaptive
 * refinement"): the state u_from of the flat forest `from` moved onto the
 * forest `to`, which shares dim, order, elems, precision, roots and extents
 * and differs from it by at most one level per block. A block of `to` that
 * is a leaf of `from` is copied; a child of a `from` leaf gets the parent
 * element's polynomial at its nodes (the prolongation I in every
 * dimension); the parent of 2^D `from` leaves gets their L2 projection in
 * the Gauss-Lobatto inner product (R = M_c^-1 I^T M_f in every dimension).
 * Both keep sum w u of each variable; coarsening brings back v's top modes,
 * so a truncated scheme truncates after it. u_from and u_to are device
 * buffers in the two forests' state layouts; stream is a cudaStream_t or
 * NULL. Synchronous. */
int twoldg_transfer(const twoldg_desc* from, const void* u_from, const twoldg_desc* to, void* u_to, void* stream);

/* The autotuner (no reference counterpart: the reference launches its
 * kernels with a fixed workgroup size). For every (dim, P, E) group of the
 * problem it times the stage kernel's launch layouts -- which kernel (the
 * register-line 3D kernel, the fixed-shape or the run-time-shape kernel),
 * threads per CTA, and one CTA per block or a persistent grid of 1 or 2
 * waves of resident CTAs -- on stages 1 to 3 of a step of size dt from u
 * (u itself is not changed), and keeps the fastest for the problem's later
 * steps. cache: NULL, or the path of a JSON file of earlier choices keyed by
 * precision, dim, P, E, metric and the block count's bit length; choices
 * found there are taken without timing and new ones are written back.
 * report (may be NULL) receives one line per group with the choice and its
 * time per stage launch in microseconds. Synchronous. */
int twoldg_autotune(twoldg_problem* p, void* u, double dt, const char* cache, char* report, size_t report_len);

/* The problem's CUDA stream (a cudaStream_t), for callers that order their
 * own work or events against the library's. */
void* twoldg_stream(twoldg_problem* p);

/* Waits for all work queued on the problem's stream. */
int twoldg_synchronize(twoldg_problem* p);

/* The right-hand side of twoldg_rhs without any device allocation, for
 * callers that cannot call cudaMalloc (a host that lends the library only
 * buffers it manages itself: a fixed arena, a pool that forbids growth, an
 * embedding runtime whose allocator must not be bypassed). No counterpart in
 * the reference. It takes the forest's descriptor instead of a problem and
 * keeps its scratch (work items, face exports, coarse-fine ghosts) in one
 * file-scope device array of 16 MiB per GPU, held until exit; a forest that
 * needs more is rejected with TWOLDG_EINVAL. The first call on a device looks
 * the array up (cudaGetSymbolAddress) and should come before any stream
 * capture. Calls share the array: calls that overlap on the GPU race.
 * Asynchronous on `stream` (a cudaStream_t; NULL is the default stream). */
int twoldg_rhs_static(const twoldg_desc* desc, void* du, const void* u, double t, void* stream);

/* ---- The particle-grid transfer (src/transfer.jl) ----
 *
 * project_source!(du, p, t, S, particles; ball, rnear, factor, var) --
 * src/transfer.jl:918-944: du[var] += factor (P S), (P S)_n = (1/w_n)
 * int_{element(n)} S phi_n, over the elements of the blocks that the
 * source's ball meets. Elements within rnear h_e of a particle take the
 * nested rule split at its support (Gauss inside, Johnston and Elliott's sinh
 * rule outside, src/transfer.jl:343-455), those within rfar h_e a graded
 * tensor Gauss rule (band by distance, :107-170), the rest the far tensor
 * Gauss rule of q = P + 3 points (:520-680). The host plans the elements and
 * the nested rule's points (projection_plan, host_elements and
 * nested_points, :984-1022, :1257-1285, :1380-1415); the device evaluates
 * and contracts. The reference's device hook for the source evaluation,
 * launch_points! (ext/TreeWaveOLDGCUDAExt.jl:23-30, src/transfer.jl:636),
 * runs a user closure at every point: here the caller either evaluates S
 * itself at the points twoldg_transfer_points lists and passes the values
 * (twoldg_project_values), or takes the built-in particle density
 * (twoldg_project_density, particle_density, src/particle.jl:117-127). */
typedef struct twoldg_particle {
    double z[3];       /* centre, physical coordinates */
    double v[3];       /* velocity, |v| < 1 */
    double ell;        /* size: the support is |L(v)(x - z)| <= ell */
    double charge;     /* Q of the built-in density source */
} twoldg_particle;

typedef struct twoldg_transfer_desc {
    const double* origins;   /* nblocks x dim: each block's origin in the particles' frame
                                (physical coordinates; ParticleFrame, src/transfer.jl:705-766) */
    const double* spacings;  /* nblocks: each block's node spacing in that frame */
    const int32_t* levels;   /* nblocks: refinement levels (the finest-level checks), or NULL */
    const uint8_t* mask;     /* nblocks: 1 for a block of the frame's patch, or NULL for all */
    double h_e;              /* the finest element width in that frame (frame_he) */
    double ball_centre[3];   /* the source's ball: elements that miss it are skipped */
    double ball_radius;
    const twoldg_particle* particles;  /* at most 8 */
    int32_t nparticles;
    double rnear;            /* nested rule within rnear h_e (0 <= rnear <= rfar) */
    /* the quadrature; 0 (or NULL) takes the reference's defaults
     * (TransferTables, src/transfer.jl:139-170) */
    int32_t q;               /* far rule points per dimension: P + 3 */
    int32_t nsinh, nmid, ninner;       /* 48, 16, 24 */
    int32_t nbands;                    /* graded bands: 4 */
    const double* band_from;           /* (1, 2, 3, 4) h_e */
    const int32_t* band_points;        /* (14, 10, 8, 7) */
    double rfar;                       /* 9 h_e */
} twoldg_transfer_desc;

typedef struct twoldg_transfer_plan twoldg_transfer_plan;

/* Plans a projection onto problem p's state (flat layout, dim 1..3): checks
 * the refusals of the reference (rnear outside [0, rfar], two supports in one
 * element, the ball or a support on a level below the finest), classifies the
 * elements and lists the nested rule's points. Synchronous. */
int twoldg_transfer_plan_create(twoldg_problem* p, const twoldg_transfer_desc* desc, twoldg_transfer_plan** out);
/* The same plan for new particle positions (and count, at most 8): the
 * ball, the frame and the quadrature are kept, as the reference's SourceBall
 * keeps them (src/transfer.jl:946-982), and only what the positions decide
 * -- the elements by rule and the nested rule's points -- is redone, into the
 * plan's device buffers. Waits for the plan's earlier projections first.
 * Synchronous. */
int twoldg_transfer_plan_update(twoldg_transfer_plan* plan, const twoldg_particle* particles, int32_t nparticles);
int twoldg_transfer_plan_destroy(twoldg_transfer_plan* plan);
/* counts[8]: far elements, far points, graded elements, graded points,
 * near elements, near points, near chunks, all points. */
int twoldg_transfer_plan_counts(const twoldg_transfer_plan* plan, int64_t* counts);
/* Every point the plan evaluates S at, as (dim, npoints) in the field type,
 * into the device array xs: the far and graded elements' Gauss points
 * element by element (dimension 1 fastest), then the nested rule's points.
 * Asynchronous on the problem's stream. */
int twoldg_transfer_points(twoldg_transfer_plan* plan, void* xs);
/* du[var] += factor P S with S's values at the listed points (a device
 * array of the field type, npoints long); var 1 (u) or 2 (v). Asynchronous. */
int twoldg_project_values(twoldg_transfer_plan* plan, const void* values, void* du, double factor, int32_t var);
/* The same with S the particles' density sum_k Q_k rho0(|L(v_k)(x - z_k)|),
 * evaluated on the device (dim 3). Asynchronous. */
int twoldg_project_density(twoldg_transfer_plan* plan, void* du, double factor, int32_t var);
/* average_shared!(ua, sn, var) -- src/transfer.jl:1616-1714, SharedNodes
 * :1520-1614: variable var (1 or 2) of the state u, in the blocks the plan's
 * ball meets, with every node that elements share replaced by the mean over
 * them (two on a face, four on an edge, eight at a corner in 3D), one
 * dimension at a time, each pair of coincident nodes across a face taking
 * their mean, the lower one's value first. A face to a block outside the
 * ball's, on another level or past the domain (no periodic images) is left
 * alone. Asynchronous on the problem's stream. */
int twoldg_average_shared(twoldg_transfer_plan* plan, void* u, int32_t var);
/* pairing(p, t, u, K, s; var, continuous) -- src/transfer.jl:1779-1797 --
 * for each of the plan's particles k with its density kernel
 * K = (grad rho_k, rho_k) (density_kernel, src/dynamic.jl:124-135; the two
 * pairings of particle_forces, src/inspiral.jl:491-504): out[4k + c] =
 * int (d rho_k / dx_c) g_h for c < 3 and int rho_k g_h for c = 3, g_h the
 * polynomial of variable var (1 or 2) of the device state u on the elements
 * that meet the support (support_elements, :1726-1758), each integrated by the
 * nested rule kept to the support. With continuous nonzero, g_h is first made
 * continuous by the mean over the elements that share each node
 * (continuous_values, :1449-1500), refused where a support element is on the
 * domain's face or next to another level. The kernel's moments int K phi_n
 * are formed in FP64 on the device at the first pairing after the particles
 * move; each pairing then gathers and sums on the device. Refused unless
 * 2 ell < h_e and the support's box lies inside the domain (no periodic
 * images); dim 3 only. Synchronous: out is host memory. */
int twoldg_pairing(twoldg_transfer_plan* plan, const void* u, int32_t var, int32_t continuous, double* out);
/* support_elements(p, s) -- src/transfer.jl:1726-1758: the elements that
 * hold a corner of particle k's support box [z - ell, z + ell], in the
 * corners' order (the first dimension fastest, the lower side first), as rows
 * (block, e0, e1, e2) of out (at most 8 rows); *n gets their number. */
int twoldg_support_elements(twoldg_transfer_plan* plan, int32_t k, int32_t* out, int32_t* n);
/* A transfer table of order P in float64 (precision 0) or float32 (1):
 * "bary" (P+1), and of the q-point Gauss-Legendre rule "gauss_nodes" (q),
 * "gauss_weights" (q), "lagrange" (q x (P+1)), "contract" ((P+1) x q); built
 * in double-double and rounded once (TransferTables, src/transfer.jl:139-170). */
int twoldg_transfer_table(int32_t order, int32_t precision, const char* name, int32_t q, void* out);

/* Batched ensemble: n independent problems stepped together, the blocks of
 * all of them as one work list per (dim, order, elems) group and up to 16
 * RK4 steps per CUDA graph launch. No reference counterpart (the reference runs
 * one forest per WaveProblem); each member behaves as twoldg_rk4_step on its
 * own problem. States are one device buffer: member k's state starts at word
 * offsets[k] (as returned by twoldg_batch_offsets). */
typedef struct twoldg_batch twoldg_batch;
int twoldg_batch_create(int32_t n, const twoldg_desc* descs, twoldg_batch** out);
int twoldg_batch_destroy(twoldg_batch* b);
int twoldg_batch_offsets(const twoldg_batch* b, int64_t* offsets, int64_t* total_words);
int twoldg_batch_rk4_step(twoldg_batch* b, void* u, const double* dt, int32_t nsteps);
/* twoldg_autotune for a batch: dt[n] per problem, one choice per shape group. */
int twoldg_batch_autotune(twoldg_batch* b, void* u, const double* dt, const char* cache, char* report,
                          size_t report_len);
int twoldg_batch_synchronize(twoldg_batch* b);
/* The batch's CUDA stream (a cudaStream_t), as twoldg_stream gives a
 * problem's. */
void* twoldg_batch_stream(twoldg_batch* b);

#ifdef __cplusplus
}
#endif

#endif /* TWOLDG_H */
