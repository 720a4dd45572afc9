/*
 * dompap_gpu.h — C ABI of the GB300 (sm_103a) molecular-dynamics hot path.
 *
 * One handle (dp_sim) holds one periodic system of N point particles in D
 * dimensions (D = 2, 3 or 4) resident in GPU memory, plus its pair potential,
 * neighbour list and integrator settings. Every entry point takes plain
 * pointers and sizes; host arrays use dompap's own layouts (row-major (N, D)
 * float64 positions etc.). Every entry point returns 0 (DP_OK) or a DP_ERR_*
 * code; dp_last_error() then describes the failure. A handle is not
 * thread-safe; distinct handles may be used from distinct threads.
 *
 * Each declaration names the dompap function it replaces (paths inside the
 * dompap project, version 0.0.6). The Python `Simulation` in dompap_gb300 is
 * the drop-in binding over these entry points (ctypes).
 */
#ifndef DOMPAP_GPU_H
#define DOMPAP_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DP_OK 0
#define DP_ERR_ARG 1        /* invalid argument / shape / state                  */
#define DP_ERR_CUDA 2       /* CUDA runtime error                                */
#define DP_ERR_NVRTC 3      /* the generated pair potential failed to compile    */
#define DP_ERR_OVERFLOW 4   /* neighbour list exceeded max_number_of_neighbors   */
#define DP_ERR_GEOMETRY 5   /* box too small for the single-image convention     */
#define DP_ERR_NONFINITE 6  /* a force or position became NaN / Inf              */
#define DP_ERR_NOPOT 7      /* no pair potential set                             */
#define DP_ERR_TIMEOUT 8    /* a bounded device-side wait gave up; that launch's
                               results are discarded, the context stays usable  */

#define DP_PREC_FP64 0 /* float64 pair arithmetic (parity mode)                        */
#define DP_PREC_FP32 1 /* float32 pair forces, float64 integration, wrap and sums      */
#define DP_PREC_MLP 2  /* float32 cheap terms + tensor-core surrogate for costly terms */

#define DP_NL_CELL 0   /* cell list + Verlet list (falls back to all pairs if < 3 cells) */
#define DP_NL_ALLPAIRS 1 /* O(N^2) build, rows in ascending index order                */

#define DP_INT_GJF 0 /* Langevin G-JF leap-frog                         */
#define DP_INT_NVE 1 /* NVE leap-frog                                   */

#define DP_PAIR_CONST 0 /* sigma, epsilon constants                              */
#define DP_PAIR_TYPES 1 /* (ntypes, ntypes) tables indexed by particle type      */
#define DP_PAIR_DENSE 2 /* (N, N) matrices sigma[n, m] (index callables)         */

typedef struct dp_sim dp_sim;

typedef struct dp_stats {
    int64_t steps;              /* integrated steps (RNG counter)                     */
    int64_t rebuilds;           /* neighbour-list builds on the device                */
    int32_t max_neighbors;      /* largest neighbour count of the current list        */
    int32_t neighbor_capacity;  /* current per-particle list capacity                 */
    int32_t cells[4];           /* cells per axis of the cell list (0: all pairs)     */
    int32_t cell_capacity;      /* particles per cell slot array                      */
    int32_t method_used;        /* DP_NL_CELL or DP_NL_ALLPAIRS                       */
    double nl_cutoff;           /* largest sigma * r_cut + skin                       */
    int32_t conditional_graphs; /* 1: run() skips the rebuild kernels on steps that need
                                   no rebuild (conditional graph nodes); 0: they are
                                   launched every step and return at once            */
    int32_t pad;
} dp_stats;

/* Last error message of the calling thread ("" if none). */
const char *dp_last_error(void);
/* ABI version (major * 10000 + minor * 100 + patch). */
int dp_version(void);

/* Create / destroy a system of n particles in dim dimensions on the current
 * CUDA device. Replaces the state arrays of dompap/Simulation.py:101-147. */
int dp_create(int dim, int64_t n, int precision, dp_sim **out);
int dp_destroy(dp_sim *sim);
int dp_set_precision(dp_sim *sim, int precision);

/* State upload / download, (N, D) row-major float64 / int32 and (N,) arrays.
 * Replaces direct assignment of Simulation.positions / velocities / betas /
 * image_positions / masses / particle_types (dompap/Simulation.py:101-114,
 * set_masses :232, set_types :292). */
int dp_set_positions(dp_sim *sim, const double *positions);
int dp_get_positions(dp_sim *sim, double *positions);
int dp_set_velocities(dp_sim *sim, const double *velocities);
int dp_get_velocities(dp_sim *sim, double *velocities);
int dp_set_betas(dp_sim *sim, const double *betas);
int dp_get_betas(dp_sim *sim, double *betas);
int dp_set_images(dp_sim *sim, const int32_t *images);
int dp_get_images(dp_sim *sim, int32_t *images);
int dp_set_masses(dp_sim *sim, const double *masses);
int dp_set_types(dp_sim *sim, const int32_t *types);
/* Box side lengths (D,). Replaces Simulation.box_vectors / scale_box
 * (dompap/Simulation.py:527-543). Forces a neighbour-list rebuild. */
int dp_set_box(dp_sim *sim, const double *box);

/* Pair potential: CUDA C++ source defining
 *   template <typename R> __device__ R dp_pair_u(R s);  (u(s) - u(r_cut))
 *   template <typename R> __device__ R dp_pair_f(R s);  (-du/ds)
 *   template <typename R> __device__ R dp_pair_c(R s);  (d2u/ds2)
 * generated from the SymPy expression by dompap_gb300.codegen; compiled with
 * NVRTC for sm_103a. Replaces make_pair_potential (dompap/potential.py:43-66)
 * and the hard-coded potentials (:10-40). Values are 0 where s > r_cut. */
int dp_set_potential(dp_sim *sim, const char *device_source, double r_cut);
/* sigma / epsilon: mode DP_PAIR_CONST (tables of 1), DP_PAIR_TYPES
 * (ntypes x ntypes) or DP_PAIR_DENSE (N x N). Replaces
 * set_pair_potential_parameters (dompap/Simulation.py:469-525). */
int dp_set_pair_params(dp_sim *sim, int mode, int ntypes, const double *sigma, const double *epsilon);
/* Skin, per-particle capacity and build method; forces a rebuild.
 * Replaces set_neighbor_list (dompap/Simulation.py:307-381). */
int dp_set_neighbor_list(dp_sim *sim, double skin, int max_neighbors, int method);
/* Rebuild if any particle moved more than skin/2 since the last build
 * (check != 0) or unconditionally (check == 0). *rebuilt (may be NULL) tells
 * which. Replaces update_neighbor_list (dompap/Simulation.py:383-401) and
 * neighbor_list_is_old (dompap/neighbor_list.py:183-201). */
int dp_update_neighbor_list(dp_sim *sim, int check, int *rebuilt);
/* Neighbour list in dompap's layout: (N, kmax) int32, rows ascending, -1
 * padded. *max_count receives the largest row length (rows longer than kmax
 * are truncated). Replaces Simulation.neighbor_list as built by
 * get_neighbor_list_double_loop (dompap/neighbor_list.py:7-39). */
int dp_get_neighbor_list(dp_sim *sim, int32_t *out, int kmax, int32_t *max_count);
/* Positions at the last neighbour-list build, (N, D) row-major.
 * Replaces Simulation.positions_neighbour_list (dompap/Simulation.py:381). */
int dp_get_reference_positions(dp_sim *sim, double *positions);

/* Integrator parameters. Replaces set_integrator (dompap/Simulation.py:739-759);
 * seed keys the counter-based normal deviates. */
int dp_set_integrator(dp_sim *sim, double time_step, double temperature, double damping_time, uint64_t seed);
/* `steps` steps of integrator `kind` (DP_INT_GJF or DP_INT_NVE). Each step:
 * neighbour-list check/rebuild, forces, integrate, wrap into box.
 * Replaces Simulation.run / step / step_leap_frog (dompap/Simulation.py:681-737)
 * with make_one_step / make_one_step_leap_frog (dompap/integrator.py:5-40)
 * and wrap_into_box (dompap/positions.py:90-98). */
int dp_run(dp_sim *sim, int64_t steps, int kind);
/* Self-test of the bounded device-side waits (no counterpart in the
 * reference): a kernel waits on an mbarrier that nothing arrives at, gives up
 * after `limit` tries (1 .. 2^20), frees the tensor memory it holds and flags
 * the failure; returns DP_ERR_TIMEOUT as a real timeout would, and the handle
 * stays usable. No GPU fault is involved. */
int dp_selftest_bounded_wait(dp_sim *sim, int32_t limit);
/* dp_run on host arrays, as dompap's step keeps its state: the (N, D)
 * float64 row-major positions, velocities and betas given (each may be NULL:
 * kept) are uploaded, `steps` steps run, and the arrays asked for (each may
 * be NULL) are written back; one call, one final wait. Replaces
 * Simulation.step / run (dompap/Simulation.py:681-737) with its NumPy state
 * arrays in and out (dompap/integrator.py:17-40 returns new arrays). Page-locked
 * host arrays are read and written by the device directly. */
int dp_run_host(dp_sim *sim, const double *positions, const double *velocities, const double *betas, int64_t steps,
                int kind, double *positions_out, double *velocities_out, double *betas_out);
/* Same as dp_run, also returning the device time of the steps in ms
 * (CUDA events on the handle's stream). */
int dp_run_timed(dp_sim *sim, int64_t steps, int kind, float *ms);

/* Forces (N, D) row-major. Replaces get_forces (dompap/Simulation.py:594-619)
 * -> _get_forces (dompap/potential.py:163-188). */
int dp_forces(dp_sim *sim, double *forces);
/* Potential energy. Replaces get_potential_energy -> _get_total_energy
 * (dompap/Simulation.py:545-570, dompap/potential.py:69-100). */
int dp_potential_energy(dp_sim *sim, double *energy);
/* Pair virial W. Replaces get_virial -> _get_virial_double_loop
 * (dompap/Simulation.py:946-967, dompap/potential.py:253-279). */
int dp_virial(dp_sim *sim, double *virial);
/* Per-particle Laplacian (N,). Replaces get_laplacian -> _get_laplacian
 * (dompap/Simulation.py:1205-1229, dompap/potential.py:327-364). */
int dp_laplacian(dp_sim *sim, double *laplacian);
/* sum_n m_n |v_n|^2. Used by get_temperature / get_kinetic_energy /
 * get_pressure (dompap/Simulation.py:817-836, 896-910, 969-988). */
int dp_sum_mv2(dp_sim *sim, double *sum_mv2);
/* u_cut, f_cut, c_cut of the compiled potential at n scaled distances
 * (the callables returned by make_pair_potential, dompap/potential.py:61-66). */
int dp_eval_potential(dp_sim *sim, const double *s, int64_t n, double *u, double *f, double *c);
/* Standard normal deviates the G-JF step `step` draws, (N, D) row-major
 * (the np.random.normal of dompap/integrator.py:30; test hook). */
int dp_get_normals(dp_sim *sim, int64_t step, double *normals);

/* Wrap positions into [0, L) and update the images in place. Replaces
 * Simulation.wrap_into_box (dompap/Simulation.py:656-679, positions.py:90-98). */
int dp_wrap(dp_sim *sim);
/* Histogram of all ordered pair distances (i of type_a, j of type_b; -1 = all;
 * self pairs included) with np.round minimum image over nbins bins with the
 * nbins + 1 ascending edges (np.histogram semantics). The host normalises as
 * get_radial_distribution_function (dompap/positions.py:58-87) does. */
int dp_rdf_counts(dp_sim *sim, int type_a, int type_b, const double *edges, int nbins, uint64_t *counts);

int dp_get_stats(dp_sim *sim, dp_stats *stats);
#define DP_KERNEL_FORCES 0  /* pair forces                                */
#define DP_KERNEL_GJF 1     /* G-JF integrate + wrap + skin test            */
#define DP_KERNEL_NVE 2     /* NVE integrate + wrap + skin test             */
#define DP_KERNEL_REBUILD 3 /* forced neighbour-list rebuild (all kernels)  */
#define DP_KERNEL_SKIN 4    /* skin test alone                              */
#define DP_KERNEL_STEP 5    /* fused step: pair forces + integrate + wrap + skin test
                               (the kernel run() launches outside the surrogate mode) */
/* Device time of `reps` back-to-back launches of one step kernel on the
 * current state (ms per launch, CUDA events on the handle's stream). The
 * integrator variants advance the state; the list is rebuilt afterwards. */
int dp_time_kernel(dp_sim *sim, int which, int reps, float *ms_per_launch);
/* sum_n m_n |v_n|^2 like dp_sum_mv2, but on caller-owned device arrays and
 * without allocating anything; it has no counterpart in the reference.
 * For callers that cannot call cudaMalloc: hosts that hand out all device
 * memory from their own pool or arena (a framework's caching allocator, a
 * memory budget fixed at start-up), where an allocation made behind their
 * back can fail once the pool holds the memory, or breaks their accounting.
 * velocities: device (N, dim) row-major float64; masses: device (N,); out:
 * device, one double; stream: a cudaStream_t (NULL = default stream).
 * Asynchronous on `stream`.
 * Scratch: a fixed 128 KiB device array inside this library (one double per
 * 256 particles), so N is at most 4,194,304; a larger N returns DP_ERR_ARG
 * before any launch. Every GPU that loads the library holds the array until
 * the process exits. The first call on a device looks up the array's device
 * address (set-up, once per device, with that device current); make that
 * first call before any stream capture. The address is kept for the life of
 * the process: after cudaDeviceReset, call nothing here again on that device.
 * Every call shares the array and overwrites the partial sums it reads, so
 * nothing carries over from the previous call; calls that overlap on the GPU
 * (different streams at once) race on it. */
int dp_sum_mv2_noalloc(const double *velocities, const double *masses, int64_t n, int dim, double *out,
                       void *stream);

/* Force and energy methods (dompap's method strings,
 * dompap/Simulation.py:126-133 and the dispatch in get_forces :594-654 and
 * get_potential_energy :545-592). DP_METHOD_LIST: the neighbour-list kernels
 * ("neighbor list", dompap/potential.py:69-100,163-188). DP_METHOD_ALLPAIRS:
 * no list, every pair evaluated ("double loop" and "vectorized" forces,
 * potential.py:217-250,298-324: F_n = sum_m eps(n,m) f(r/sigma(n,m)) d/r;
 * "double loop" energies, :103-160: U = sum_{n<m} eps(n,m) u(r/sigma(n,m))).
 * DP_METHOD_ALLPAIRS_NEWTON (forces only): "double loop single core"
 * (:191-214), every pair with the parameters of (min(n,m), max(n,m)); equal
 * to the others unless sigma/epsilon are asymmetric callables. run() with an
 * all-pairs force method keeps no list (the list is built on demand for the
 * observables that use it). The surrogate mode always uses its list kernels. */
#define DP_METHOD_LIST 0
#define DP_METHOD_ALLPAIRS 1
#define DP_METHOD_ALLPAIRS_NEWTON 2
int dp_set_pair_methods(dp_sim *sim, int force_method, int energy_method);
/* Launch shape of the fused step kernel, chosen by the autotuner
 * (dompap/tools/autotune.py:112-162 times dompap's force methods on the
 * actual system; here the candidates are launch shapes of the one GPU step):
 * lanes per particle 1 (one thread per particle), 4 or 32 (the particle's
 * list split over a lane group), 0 = by system size (32 up to 8,192
 * particles, 4 up to 65,536, else 1); blocks_per_sm = resident 256-thread
 * CTAs per SM the step is compiled for (1..8; 0 = the default of the mode;
 * a change recompiles the pair program). dp_get_step_launch reports the shape
 * in use. */
int dp_set_step_launch(dp_sim *sim, int lanes, int blocks_per_sm);
int dp_get_step_launch(dp_sim *sim, int *lanes, int *blocks_per_sm);
/* Number of kernels the last dp_run launched (graph nodes included). */
int64_t dp_kernel_launches(dp_sim *sim);

/* ---------------------------------------------------------------------------
 * Batched replicas: many independent periodic systems (sizes up to 65535,
 * each with its own box and temperature) advanced by one persistent kernel
 * per run (captured in a CUDA graph); float32 pair forces from fixed-point
 * displacements, float64 G-JF / NVE integration and wrap. sigma = epsilon = 1.
 * Replaces a Python loop of Simulation.run over replicas
 * (dompap/Simulation.py:726-737 per replica).
 * ------------------------------------------------------------------------- */
typedef struct dp_batch dp_batch;
/* counts: (n_rep,) particles per replica; particles are stored replica after replica. */
int dp_batch_create(int dim, int n_rep, const int32_t *counts, dp_batch **out);
int dp_batch_destroy(dp_batch *batch);
/* positions, velocities: (sum N, D) row-major; boxes: (n_rep, D); temperatures: (n_rep,).
 * Positions must lie in [0, L) of their replica. */
int dp_batch_set_state(dp_batch *batch, const double *positions, const double *velocities, const double *boxes,
                       const double *temperatures);
/* Any of the outputs may be NULL. images: (sum N, D) int32. */
int dp_batch_get_state(dp_batch *batch, double *positions, double *velocities, int32_t *images);
/* Generated pair potential (as dp_set_potential), compiled for the batch kernel. */
int dp_batch_set_potential(dp_batch *batch, const char *device_source, double r_cut);
int dp_batch_set_integrator(dp_batch *batch, double time_step, double damping_time, double mass, uint64_t seed);
/* Replicas with more than split_n particles run with threads_large threads per
 * CTA, the others with threads_small (128, 256, 512 or 1024): the tile shape
 * the autotuner picks. */
int dp_batch_set_launch(dp_batch *batch, int split_n, int threads_small, int threads_large);
/* `steps` steps of every replica (nve: leap-frog instead of G-JF). Every
 * sample_every steps (0: never) U, W and sum m v^2 of each replica are added
 * to its observables. record_forces keeps the last step's float32 forces.
 * ms (may be NULL) receives the device time. */
int dp_batch_run(dp_batch *batch, int64_t steps, int sample_every, int nve, int record_forces, float *ms);
/* Compile the pair program of (dim, precision, pair mode, batch kernels) for
 * a generated potential with NVRTC and discard it: a host-only check of the
 * device code (no GPU needed; no counterpart in the reference). cubin_bytes
 * (may be NULL) receives the CUBIN size. */
int dp_nvrtc_check(int dim, int precision, int pair_mode, int with_batch, const char *device_source,
                   int64_t *cubin_bytes);
/* The same compile with the assembler's verbose report: registers, spill
 * stores/loads and shared memory of every kernel of the program, written to
 * log (NUL-terminated, truncated to log_capacity); log_bytes (may be NULL)
 * receives the full length. Host only (no counterpart in the reference). */
int dp_nvrtc_resources(int dim, int precision, int pair_mode, int with_batch, const char *device_source, char *log,
                       int64_t log_capacity, int64_t *log_bytes);
/* Verlet lists for the batch (replaces the per-step 27-cell stencil; no
 * counterpart in the reference, whose replicas each run dompap's own list,
 * dompap/neighbor_list.py:7-201): partners within r_cut + skin, rebuilt per
 * replica when a particle moved more than skin/2 and at the start of every
 * run. kmax = 0 sizes the lists from the densest replica; a replica whose list
 * would overflow uses the stencil for the rest of that run. skin < 0 turns the
 * lists off. Default: skin 0.45, kmax 0. */
int dp_batch_set_neighbor_list(dp_batch *batch, double skin, int kmax);
/* List builds and overflowed replicas since creation, and the list capacity in use. */
int dp_batch_list_stats(dp_batch *batch, int64_t *builds, int64_t *overflowed, int32_t *kmax);
/* (n_rep, 4): sum of U, sum of W, sum of sum m v^2, number of samples. reset != 0 zeroes them. */
int dp_batch_observables(dp_batch *batch, double *out, int reset);
/* (sum N, D) forces of the last recorded step (float32 values). */
int dp_batch_last_forces(dp_batch *batch, double *forces);

/* ---------------------------------------------------------------------------
 * Pair surrogate: a 1 -> 64 -> 64 -> 2 tanh network of s = r^2 giving
 * (u, f r) of the costly terms of a pair potential, bf16 weights and fp32
 * accumulation on tensor cores (mma.sync m16n8k16), trained by the library's
 * own forward/backward kernels with Adam. No counterpart in dompap (it
 * evaluates every term through its jitted SymPy lambdas,
 * dompap/potential.py:43-66); the codegen path is its fallback and yardstick.
 * Parameters (fp32, dp_mlp_param_count() of them): w1[64], b1[64],
 * W2[64][64] (row = output unit), b2[64], W3[2][64], b3[2]; norm[4]:
 * x_mean, 1/x_scale (x = (s - x_mean)/x_scale), u_scale, f_scale (of f r).
 * ------------------------------------------------------------------------- */
typedef struct dp_mlp dp_mlp;
int dp_mlp_create(dp_mlp **out);
int dp_mlp_destroy(dp_mlp *mlp);
int dp_mlp_param_count(void);
int dp_mlp_set_params(dp_mlp *mlp, const float *params, const float *norm);
int dp_mlp_get_params(dp_mlp *mlp, float *params);
/* Training set: n inputs s (float) and normalised targets (n, 2). */
int dp_mlp_set_data(dp_mlp *mlp, const float *s, const float *targets, int64_t n);
/* `steps` Adam steps on random minibatches of `batch` samples, learning rate
 * decaying (cosine) from lr0 to lr1; loss (y0-t0)^2 + wf (y1-t1)^2. accurate
 * selects the software tanh (else the hardware approximation, as inference
 * uses). losses (may be NULL) receives the minibatch loss of every step. */
int dp_mlp_train(dp_mlp *mlp, int64_t steps, int batch, float lr0, float lr1, float wf, uint64_t seed, int accurate,
                 float *losses);
/* Network outputs y (n, 2) for inputs s. */
int dp_mlp_eval(dp_mlp *mlp, const float *s, int64_t n, float *y, int accurate);
/* Gradient (dp_mlp_param_count() floats) and mean loss of a batch. */
int dp_mlp_gradients(dp_mlp *mlp, const float *s, const float *targets, int64_t n, float wf, int accurate,
                     float *grad, float *loss);
/* Use `mlp` for the costly terms in the pair kernels of `sim` (the potential
 * set with dp_set_potential is then the cheap remainder, with the full
 * potential's shift). The network must outlive its use; NULL detaches. */
int dp_set_mlp(dp_sim *sim, dp_mlp *mlp);

#ifdef __cplusplus
}
#endif
#endif /* DOMPAP_GPU_H */
