/*
 * mtg.h - C ABI of the GB300 engine for MADDY's Brownian/Langevin hot path
 * (6-DOF coarse-grained tubulin beads: forces, pair lists, Euler-Maruyama
 * update with HybridTaus noise, energies, TEA hydrodynamics).
 *
 * Every function returns an int status: MTG_OK (0) or a negative MTG_E_*
 * code; mtg_last_error_string() describes the last failure of the calling
 * thread.  Host buffers are plain pointers owned by the caller; device
 * buffers are owned by the engine.  One engine = one CUDA stream; an engine
 * is not thread-safe, distinct engines are independent.
 *
 * Reference interfaces replaced (paths inside the klyshko/MT project):
 *   compute(Coord*, Coord*, Parameters&, Topology&, Energies*)   src/compute_cuda.cuh:17
 *   initIntegration / deleteIntegration                          src/compute_cuda.cuh:18-19
 *   initTeaIntegrator / updateTea / integrateTea / deleteTea...  src/bdhitea.cuh:18-24
 *   initRand(int seed, int Np)                                   src/ht.cuh:14
 * The engine entry points below are what a compute() drop-in calls; see
 * mt_gb300/host/mtg_compute.cpp for that drop-in.
 */
#ifndef MTG_H_
#define MTG_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define MTG_OK            0
#define MTG_E_CUDA       -1  /* a CUDA runtime call failed (reference: checkCUDAError -> die, src/Cuda.h:120-135) */
#define MTG_E_CONFIG     -2  /* invalid parameters, sizes or call arguments (reference: DIE, src/configreader.cpp:129) */
#define MTG_E_OVERFLOW   -3  /* a neighbour list exceeded its capacity (reference: silent overflow, src/compute_cuda.cu:1076) */
#define MTG_E_NONFINITE  -4  /* a non-finite energy total (reference: prints, src/updater.cpp:27-30) */
#define MTG_E_TEA_EPS    -5  /* TEA epsilon > 1 in capricious mode, > epsmax, or a too-diagonal tensor (reference: exit(-1), src/bdhitea.cu:89-106) */
#define MTG_E_TIMEOUT    -6  /* a bounded device-side wait gave up */
#define MTG_E_STATE      -7  /* call out of sequence (e.g. surrogate not trained) */

/* Coord as laid out by the reference (src/mt.h:63-71): 7 floats per bead in
 * the order x, y, z, fi, theta, psi, w (w unused).  Host state buffers of
 * this ABI use that AoS layout so a caller can pass its Coord* directly. */
#define MTG_COORD_FLOATS 7

/* Energies as laid out by the reference (src/mt.h:94-102): 7 doubles in the
 * order U_harm, U_long, U_lat, U_psi, U_fi, U_teta, U_lj. */
#define MTG_ENERGY_TERMS 7

/* Scalar parameters of the hot path.  Each field carries the meaning (and
 * units: nm, ps, kcal/mol, K) of the Parameters field of the same name,
 * src/parameters.h:246-318; derived values (gammaR, gammaTheta, varR,
 * varTheta) are computed by the caller exactly as src/preparator.cpp:209-221
 * does, see mtg_derive_params(). */
typedef struct {
    float dt, Temp, viscosity;
    float gammaR, gammaTheta, varR, varTheta;
    float alpha, freeze_temp;
    /* harmonic bond and bending (src/parameters.h:270-278) */
    float C, B_psi, B_fi, B_theta, psi_0, fi_0, theta0_gtp, theta0_gdp;
    /* Morse longitudinal / lateral (src/parameters.h:279-283) */
    float A_lat, A_long, D_lat, D_long, seam_coeff;
    /* Gaussian barriers (src/parameters.h:296-302); w_* already divided by 2*sqrt(-2 ln 0.5) */
    int barrier;
    float a_barr_long, r_barr_long, w_barr_long, a_barr_lat, r_barr_lat, w_barr_lat;
    /* LJ repulsion and list (src/parameters.h:304-308) */
    int lj_on;
    float ljscale, ljsigma6, ljpairscutoff;
    int ljpairsupdatefreq;
    /* cylindrical walls (src/parameters.h:290-295); per-trajectory zs passed in the topology */
    int is_wall;
    float rep_r, rep_eps, rep_leftborder;
    /* assembly mode: pair lists rebuilt on device (src/parameters.h:255) */
    int is_assembly;
    /* TEA hydrodynamics (Tea, src/mt.h:104-121; keys src/parameters.h:236-242) */
    int hdi_on;
    float tea_a;
    int tea_epsilon_freq;
    int tea_capricious;
    float tea_epsmax;
    /* HybridTaus seed (src/parameters.h:248) */
    int rseed;
    /* CUDA device of the engine (Parameters::device, src/parameters.h:263;
     * the reference calls cudaSetDevice(par.device) in initIntegration) */
    int device;
} mtg_params;

/* Topology of a uniform batch, in the reference's layout (Topology,
 * src/mt.h:73-92): Ntr trajectories of Ntot beads; per-template arrays
 * ([Ntot]) are shared by all trajectories, per-bead arrays are [Ntot*Ntr]
 * with bead p = ind + traj*Ntot.  Longitudinal/lateral lists are read only
 * when is_assembly == 0 (static lists, src/preparator.cpp:357-560). */
typedef struct {
    int Ntot, Ntr;
    int maxHarmonicPerMonomer;
    const int *harmonicCount;        /* [Ntot] */
    const int *harmonic;             /* [maxHarmonicPerMonomer*Ntot], sign-encoded */
    int maxLongitudinalPerMonomer;   /* list capacity (reference: 8, src/preparator.cpp:722) */
    const int *longitudinalCount;    /* [Ntot*Ntr] or NULL */
    const int *longitudinal;         /* [maxLong*Ntot*Ntr] or NULL */
    int maxLateralPerMonomer;        /* list capacity (reference: 16, src/preparator.cpp:721) */
    const int *lateralCount;
    const int *lateral;
    int maxLJPerMonomer;             /* list capacity (reference: 256, src/compute_cuda.cu:1076) */
    const uint8_t *fixed;            /* [Ntot] */
    const int *mon_type;             /* [Ntot] 0 = alpha, 1 = beta */
    const uint8_t *extra;            /* [Ntot*Ntr] */
    const int *gtp;                  /* [Ntot*Ntr] */
    const int *on_tubule_cur;        /* [Ntot*Ntr] */
    const float *zs;                 /* [Ntr] wall height per trajectory (Parameters::zs) */
} mtg_topology;

/* Topology of a ragged batch: trajectory t owns beads offsets[t] ..
 * offsets[t+1]-1.  All per-bead arrays have offsets[ntraj] entries; list and
 * harmonic indices are local to the bead's trajectory and use the reference's
 * sign encoding.  No reference counterpart (the reference batches only
 * uniform copies of one PDB, src/preparator.cpp:303-317). */
typedef struct {
    int ntraj;
    const int *offsets;              /* [ntraj+1] */
    int maxHarmonicPerMonomer;
    const int *harmonicCount;        /* [nbeads] */
    const int *harmonic;             /* [maxHarmonicPerMonomer*nbeads] bead-major */
    int maxLongitudinalPerMonomer, maxLateralPerMonomer, maxLJPerMonomer;
    const int *longitudinalCount;    /* [nbeads] or NULL (assembly mode) */
    const int *longitudinal;         /* [maxLong*nbeads] bead-major or NULL */
    const int *lateralCount;
    const int *lateral;
    const uint8_t *fixed;            /* [nbeads] */
    const uint8_t *extra;            /* [nbeads] */
    const int *mon_type;             /* [nbeads] */
    const int *gtp;                  /* [nbeads] */
    const int *on_tubule_cur;        /* [nbeads] */
    const float *zs;                 /* [ntraj] */
} mtg_batch_topology;

typedef struct mtg_engine mtg_engine;

/* Last error message of the calling thread (never NULL). */
const char *mtg_last_error_string(void);

/* Fills gammaR, gammaTheta, varR, varTheta from dt, Temp, viscosity, hdi_on
 * and tea_a as src/preparator.cpp:209-219 does (k_B = 0.0019872041 kcal/mol/K,
 * r_mon = 2 nm). */
int mtg_derive_params(mtg_params *p);

/* Creates an engine for a uniform batch (replaces initIntegration,
 * src/compute_cuda.cu:977-1098, and initTeaIntegrator, src/bdhitea.cu:13-35).
 * Seeds the HybridTaus streams from p->rseed as initRand(rseed, 2*Ntot*Ntr)
 * does (src/HybridTaus.cu:21-48).  The state must be uploaded before stepping. */
int mtg_create(const mtg_params *p, const mtg_topology *top, mtg_engine **out);

/* Creates an engine for a ragged batch (no reference counterpart). */
int mtg_create_batch(const mtg_params *p, const mtg_batch_topology *top, mtg_engine **out);

/* Frees every device buffer of the engine (replaces deleteIntegration,
 * src/compute_cuda.cu:1100-1123, and deleteTeaIntegrator, src/bdhitea.cu:44-55). */
int mtg_destroy(mtg_engine *e);

int mtg_num_beads(const mtg_engine *e, int *nbeads, int *ntraj);

/* Re-seeds all 2*nbeads HybridTaus streams with the reference's ran2-based
 * generator (src/HybridTaus.cu:32-48, src/ran2.h:18-56). */
int mtg_seed_rng(mtg_engine *e, int rseed);
/* The HybridTaus states of nstreams streams (4*nstreams uint32) as
 * generateSeeds makes them from rseed (src/HybridTaus.cu:32-48), on the host
 * only: how a batch split over several engines gets the streams one engine
 * of the whole batch would have (stream g and g + nbeads of each bead). */
int mtg_generate_seeds(int rseed, long long nstreams, uint32_t *seeds);
/* Reads / writes the raw HybridTaus states, 2*nbeads uint4 = 8*nbeads uint32
 * (stream p drives xyz noise of bead p, stream p+nbeads its angle noise). */
int mtg_download_rng(mtg_engine *e, uint32_t *seeds);
int mtg_upload_rng(mtg_engine *e, const uint32_t *seeds);

/* Bit-exact restart.  Extends writeRestart / readRestart
 * (src/preparator.cpp:664-714), which keep the coordinates as "%f" text and
 * re-seed the noise, with one binary file that holds everything a resumed run
 * needs to reproduce the uninterrupted run bit for bit: the bead state in
 * full precision, both HybridTaus streams of every bead, the per-bead flags
 * (gtp / extra / on_tubule), the neighbour lists of the current pair-list
 * period and the TEA state (C_i row sums, beta, epsilon).  `step` is the next
 * step to run.  Reading checks the file's hash and that it belongs to a system
 * of the same sizes and modes (MTG_E_CONFIG otherwise); the learned-TEA
 * re-check state is not part of it. */
int mtg_write_restart(mtg_engine *e, const char *path, long long step);
int mtg_read_restart(mtg_engine *e, const char *path, long long *step);

/* Stride-step outputs without stalling the step loop.  Replaces the
 * synchronous download of r at stride steps (src/compute_cuda.cu:1177) with
 * saveCoordDCD (src/preparator.cpp:582-602) and OutputAllEnergies
 * (src/updater.cpp:3-43): mtg_output_open writes the DCD headers of every
 * trajectory's coordinate and angle files as createDCD + dcdWriteHeader do
 * (src/dcdio.cpp:16-154, no unit cell; remark2 NULL = the reference's
 * "REMARKS DATE: <asctime>"; energy_path NULL = standard output, else the
 * energy lines are appended to that file); mtg_output_frame queues the current state
 * and/or the energy totals: the state is converted on the engine's stream,
 * copied to pinned memory on a copy stream, and a host thread appends the
 * frames (dcdWriteFrame's layout; (x, y, z) and (fi, psi, theta)) and prints
 * the reference's energy lines, while the caller keeps stepping.  Two frames
 * can be in flight; a third request waits for the older one.
 * mtg_output_flush waits for all queued output; mtg_output_close flushes
 * and stops the writer (mtg_destroy closes an open output).  No reference
 * counterpart for the asynchronous pipeline; the bytes are the reference's. */
int mtg_output_open(mtg_engine *e, const char *const *xyz_paths, const char *const *ang_paths, int nfile, int npriv,
                    int nsavc, float delta, const char *remark2, const char *energy_path);
int mtg_output_frame(mtg_engine *e, long long step, int frame, int energies);
int mtg_output_flush(mtg_engine *e, long long *frames_written);
int mtg_output_close(mtg_engine *e);

/* Host <-> device state, Coord AoS (MTG_COORD_FLOATS floats per bead).  The
 * upload does not wrap angles; the reference wraps them once on the host in
 * initIntegration (src/compute_cuda.cu:1004-1010) and so does the compute()
 * drop-in.  Download writes r (may be NULL) and the forces of the last force
 * evaluation f (may be NULL; zero where the reference's d_f would be zero). */
int mtg_upload_state(mtg_engine *e, const float *r);
int mtg_download_state(mtg_engine *e, float *r, float *f);
/* Forces kept by plain (no-HI) steps: by default the fused step does not
 * store them (the reference zeroes d_f after integrating, src/compute_cuda.cu:966-972);
 * keep != 0 makes every step store the forces it integrated with. */
int mtg_set_keep_forces(mtg_engine *e, int keep);

/* Host-side topology changes made by the updater hooks (reference: H2D of
 * gtp src/compute_cuda.cu:1157, on_tubule_cur :1190, extra :1202). */
int mtg_set_gtp(mtg_engine *e, const int *gtp);
int mtg_set_extra(mtg_engine *e, const uint8_t *extra);
int mtg_set_on_tubule(mtg_engine *e, const int *on_tubule_cur);
/* Reads the per-bead flags back (each output may be NULL). */
int mtg_download_flags(mtg_engine *e, int *gtp, uint8_t *extra, int *on_tubule_cur, int *on_tubule_prev);

/* Stride-step analytics of the updater on the device-resident state, so a
 * stride step does not download the coordinates for them.
 *
 * mtg_mt_length: mt_length (src/updater.cpp:154-227).  A bead is on the
 * tubule when |(x, y)| < R_MT + R_THRES, |(x, y)| > 1 and cos(theta) >
 * cos(ANG_THRES) (src/mt.h:23-30); sets on_tubule_cur of every bead (after
 * copying it to on_tubule_prev when save_prev != 0, as the reference's
 * compute loop does at stride steps after the first, src/compute_cuda.cu:1186)
 * and writes the per-trajectory counts mt_len[ntraj] (may be NULL). */
int mtg_mt_length(mtg_engine *e, int save_prev, int *mt_len);
/* hydrolyse (src/updater.cpp:229-257) in two calls.  The reference draws
 * prob = rand() / RAND_MAX for every candidate dimer - GTP, not extra, on the
 * tubule now and at the previous stride - in the order dimer index (outer),
 * trajectory (inner), and hydrolyses it when prob < 0.02; afterwards every
 * GDP dimer off the tubule now and before returns to GTP.
 * mtg_hydrolysis_candidates counts the candidates; the caller draws that many
 * numbers in the reference's order and passes them to mtg_hydrolyse, which
 * applies both loops on the device.  events (may be NULL) receives one byte
 * per slot k * ntraj + t (dimer k of trajectory t; mtg_hydrolysis_slots gives
 * the number of dimer indices): 0 nothing, 1 hydrolysed, 2 back to GTP.  No
 * reference counterpart for the split; the effect is the reference's. */
int mtg_hydrolysis_candidates(mtg_engine *e, int *count);
int mtg_hydrolyse(mtg_engine *e, const double *prob, int n, int8_t *events, int *n_hydrolysed, int *n_restored);
int mtg_hydrolysis_slots(const mtg_engine *e, int *max_dimers);
/* change_conc support (src/updater.cpp:97-152): the extra beads of every
 * trajectory, and a scatter update of a few beads' state (Coord AoS) and
 * extra flags, for the dimers it re-inserts (its rand() stays with the caller). */
int mtg_count_extra(mtg_engine *e, int *n_extra);
int mtg_set_beads(mtg_engine *e, const int *idx, const float *coords, const uint8_t *extra, int n);

/* Rebuilds the LJ list (LJ_kernel, src/compute_cuda.cu:913-940) and, in
 * assembly mode, the longitudinal and lateral lists (pairs_kernel,
 * src/compute_cuda.cu:527-674) from the current state. */
int mtg_rebuild_pairs(mtg_engine *e);
/* Copies the lists to the host in the reference's layout: counts [nbeads],
 * entries [cap*nbeads] bead-major (cap = the engine's list capacity).  Any
 * pointer may be NULL. */
int mtg_download_lists(mtg_engine *e, int *lj_count, int *lj, int *long_count, int *lon,
                       int *lat_count, int *lat);
int mtg_list_capacity(const mtg_engine *e, int *max_long, int *max_lat, int *max_lj);
/* How the lists are rebuilt; both produce identical lists.  0 = automatic
 * (cell list when a trajectory has >= 512 beads), 1 = brute-force shared-memory
 * tiles over each trajectory (the reference's O(N^2) loops), 2 = per-trajectory
 * spatial-hash cell list (list capacities up to 16 longitudinal / 32 lateral). */
int mtg_set_list_method(mtg_engine *e, int method);
int mtg_get_list_method(mtg_engine *e, int *method);

/* Evaluates the forces of the current state (compute_kernel,
 * src/compute_cuda.cu:32-525) without integrating, and copies them to f
 * (Coord AoS, may be NULL). */
int mtg_compute_forces(mtg_engine *e, float *f);

/* Runs steps first_step .. first_step+nsteps-1 of the reference step loop
 * (src/compute_cuda.cu:1137-1238) without its host I/O: a pair-list rebuild
 * when step % ljpairsupdatefreq == 0, the forces, then either the
 * Euler-Maruyama update (integrate_kernel, :943-975) or, with hdi_on, the TEA
 * update (updateTea + integrateTea, src/bdhitea.cu:37-118).  When
 * mtg_rebuild_pairs() was called after the last step, the rebuild due at
 * first_step is not repeated, so a caller can rebuild, run its host hooks and
 * then step: the reference's order within a step (src/compute_cuda.cu:1140-1228).
 * Launches are replayed from CUDA graphs (one per pair-list period); the call
 * waits for them and reports device error flags. */
int mtg_step(mtg_engine *e, long long first_step, int nsteps);
/* Waits for the engine's stream and reports any device error flag. */
int mtg_sync(mtg_engine *e);

/* Energies of the current state (energy_kernel, src/compute_cuda.cu:676-911,
 * each term halved per bead).  per_bead: [nbeads*7] doubles (may be NULL),
 * per_traj: [ntraj*7] doubles summed on the device in FP64 (the reference
 * sums on the host in double, src/updater.cpp:16-26).  Returns
 * MTG_E_NONFINITE when a harm/long/lat/lj total is not finite (totals are
 * still written). */
int mtg_energies(mtg_engine *e, double *per_bead, double *per_traj);

/* TEA: recomputes the per-bead coupling sums and, in FP64 on the device,
 * epsilon and beta of every trajectory (integrateTea_epsilon_unlisted,
 * src/bdhitea_kernel.cu:84-101, and the host reduction of updateTea,
 * src/bdhitea.cu:57-118).  eps_out [ntraj] doubles and beta_out [ntraj]
 * floats may be NULL.  ci_out [nbeads*4] floats (may be NULL): the per-bead
 * row sums of squared normalised tensor entries (d_ci). */
int mtg_tea_update(mtg_engine *e, double *eps_out, float *beta_out, float *ci_out);

/* Per-trajectory energy totals written to device memory, allocating nothing.
 * No counterpart in the reference.  For callers that must not allocate at
 * the moment they ask for energies: analysis hooks running while other
 * engines on the same GPU have work in flight (cudaMalloc/cudaFree may
 * synchronise the whole device and stall that work), and processes whose
 * device memory is reserved up front by a pool allocator, where a new
 * cudaMalloc can fail.  d_per_traj: device memory for [ntraj*7] doubles
 * (the totals of mtg_energies).  The block partial sums live in a fixed
 * device array of 16384 x 7 doubles (917,504 bytes, held by every GPU that
 * loads the library until the process exits), so a batch may span at most
 * 16384 chunks of 128 beads (each trajectory is chunked separately; up to
 * 2,097,152 beads); larger batches get MTG_E_CONFIG.  The first call on
 * each engine looks up that array's device address in the engine's context
 * and keeps it in the engine (make that first call before any stream
 * capture).  Every call on a device shares the array: calls whose work
 * overlaps on the GPU (engines on different streams of the same device)
 * race and must be serialised by the caller.  Work is enqueued on the
 * engine's stream; mtg_sync() waits for it and reports a non-finite total.
 * The caller's current device is restored before the call returns; a CUDA
 * error already pending on the calling thread is reported as MTG_E_CUDA and
 * left in place, and nothing is launched. */
int mtg_energies_noalloc(mtg_engine *e, double *d_per_traj);

/* ---- learned TEA ------------------------------------------------------- */
/* A small network (32 -> 128 -> 128 -> 128 -> 4, SiLU; BF16 weights and
 * activations, FP32 accumulation on the tensor cores; Adam on FP32 master
 * weights) that predicts each bead's TEA coefficients C_i (3 components) and
 * its trajectory's beta from a 32-feature neighbourhood descriptor, so the
 * O(N^2) epsilon pass (src/bdhitea_kernel.cu:84-101, src/bdhitea.cu:57-118)
 * is skipped.  No reference counterpart. */
typedef struct mtg_surrogate mtg_surrogate;
#define MTG_SURROGATE_FEATURES 32
#define MTG_SURROGATE_OUTPUTS 4
#define MTG_SURROGATE_PARAMS 37764   /* weights and biases, see mtg_surrogate_get_params */
int mtg_surrogate_create(int device, int seed, mtg_surrogate **out);
int mtg_surrogate_destroy(mtg_surrogate *s);
/* params [MTG_SURROGATE_PARAMS] = w1[128][32], w2[128][128], w3[128][128],
 * w4[4][128], b1[128], b2[128], b3[128], b4[4] (FP32 masters);
 * norm [72] = feature means[32], feature inverse std[32], target means[4],
 * target std[4].  Either pointer may be NULL. */
int mtg_surrogate_get_params(mtg_surrogate *s, float *params, float *norm);
int mtg_surrogate_set_params(mtg_surrogate *s, const float *params, const float *norm);
/* Fits the normalisation to (X [n*32] raw features, T [n*4] targets), then
 * trains with Adam (mini-batches of `batch`, a multiple of 32; samples
 * shuffled per epoch with `seed`).  loss_per_epoch [epochs] (may be NULL):
 * mean squared error in normalised target units. */
int mtg_surrogate_train(mtg_surrogate *s, const float *X, const float *T, int n, int epochs, int batch, float lr,
                        int seed, float *loss_per_epoch);
/* Y [n*4] = predictions in target units for raw features X [n*32]. */
int mtg_surrogate_predict(mtg_surrogate *s, const float *X, int n, float *Y);
/* Loss (normalised units) and parameter gradient [MTG_SURROGATE_PARAMS] of
 * one batch, without an update (for gradient checks). */
int mtg_surrogate_loss_grad(mtg_surrogate *s, const float *X, const float *T, int n, double *loss, float *grad);
/* Descriptors X [nbeads*32] of the current state and, with TEA on, the
 * exact targets T [nbeads*4] = (C_i, beta) from a fresh epsilon pass. */
int mtg_tea_training_data(mtg_engine *e, float *X, float *T);
/* Puts the surrogate in charge of C_i and beta (s == NULL: exact TEA again).
 * Every recheck_every steps (0: never) the exact pass runs beside it and the
 * effective TEA forces of both, under identical forces and random forces,
 * are compared; when their RMS difference relative to the exact ones
 * exceeds max_err the engine falls back to exact TEA for good. */
int mtg_set_surrogate(mtg_engine *e, mtg_surrogate *s, int recheck_every, float max_err);
/* Polls of each bounded wait of the surrogate's tensor-core inference for
 * the MMAs of a layer: polls < 0 restores the default (2^20); 0 makes every
 * such wait give up at once (a test of the timeout path).  A wait that runs out ends the
 * call with MTG_E_TIMEOUT (mtg_surrogate_predict, or the mtg_step whose
 * learned-TEA work it was) instead of blocking: the kernel records the
 * timeout, waits up to the default limit for the MMAs it already issued,
 * frees its tensor memory and returns, and the next call runs normally.
 * Takes effect for step graphs captured after the call.  The reference has
 * no bounded wait: its CUDA errors end the program (src/Cuda.h:120-135). */
int mtg_surrogate_set_wait_limit(mtg_surrogate *s, int polls);
/* fell_back: 1 after a fall-back; rechecks: re-checks done; last_error: the
 * last re-check's RMS relative difference. */
int mtg_surrogate_status(mtg_engine *e, int *fell_back, int *rechecks, double *last_error);

/* Far field of the learned mode's mobility product.  No reference
 * counterpart: the reference sums T_ij over all pairs of a trajectory at
 * every step (src/bdhitea_kernel.cu:174-180) and declares, but does not
 * build, a listed variant (src/mt.h:118).  With on != 0, while the surrogate
 * is in charge (mtg_set_surrogate), each trajectory's non-extra beads are
 * arranged in a k-d tree (bisection of the current positions) with leaves of
 * at most 32 beads; pairs in leaves near each other are summed exactly as
 * the exact product does, and a node well separated from another (centres
 * farther apart than (r_N + r_J + 2 nm) / theta' and spheres more than
 * 4a + 2 nm apart, r the nodes' radii, theta' = theta for two leaves and
 * 0.7 theta otherwise), at the coarsest level where it is, acts on it through
 * 8 interpolation points per node (trilinear Chebyshev proxies of its
 * bounding box, recomputed every step), in place of its beads.  The exact re-check of
 * the learned mode then compares this product (with the surrogate's C_i and
 * beta) against the exact one, and the fall-back to exact TEA covers both.
 * theta in (0, 1]: smaller is more accurate and slower.  refresh_every: the
 * grouping is rebuilt on the host from the current positions every that many
 * steps (0: only here), before the step that reaches it. */
int mtg_set_tea_farfield(mtg_engine *e, int on, float theta, int refresh_every);
/* The grouping's leaves, the bead pairs summed exactly per step, and the
 * proxy pairs evaluated per step (zeros while off). */
int mtg_tea_farfield_stats(mtg_engine *e, int *nleaves, long long *near_pairs, long long *proxy_pairs);
/* The tree: sizes[5] = leaves, beads in leaves, near entries, nodes, far
 * entries; leaf_start [leaves+1] into leaf_bead (bead indices, leaf after
 * leaf); near_start [leaves+1] into near (leaf indices); node_range
 * [2*nodes] the begin and end of each node in leaf_bead (nodes 0 .. leaves-1
 * are the leaves); node_parent [nodes] (-1 for a root); far_start [nodes+1]
 * into far (node indices).  Call with NULL arrays for the sizes first. */
int mtg_tea_farfield_layout(mtg_engine *e, int *sizes, int *leaf_start, int *leaf_bead, int *near_start,
                            int *near, int *node_range, int *node_parent, int *far_start, int *far);
/* Effective TEA forces f_i = F_i + C_i o R_i + sum_j T_ij (F_j + beta C_i o R_j)
 * (the x, y, z of [nbeads*4]) of the current state with the engine's current
 * C_i and beta, from one force evaluation and one draw of random forces:
 * feff_exact by the all-pairs product, feff_ff by the far-field one (needs
 * the far field on); rforce [nbeads*4] receives the random forces.  Any
 * pointer may be NULL.  The pair lists are rebuilt from the current state
 * first.  The draw advances the noise streams g as a step's does.  No
 * reference counterpart (for checks of the approximation). */
int mtg_tea_effective_forces(mtg_engine *e, float *feff_exact, float *feff_ff, float *rforce);

/* ---- tuning ------------------------------------------------------------ */
/* Launch shapes of the engine's kernels.  list_method as
 * mtg_set_list_method (1 tiles, 2 cells); step_block: threads per CTA of the
 * fused plain step (64, 128, 256); tea_slices: threads per bead in the
 * all-pairs TEA kernels (1, 2, 4, 8); tea_jparts: parts the j range of a
 * work item is split into (1, 2, 3, 4).  With more than one part, the items
 * of the last one to two waves of a launch (all items of a launch shorter
 * than two waves) run as that many shorter CTAs, so the last waves are
 * fuller; the parts' sums meet in a second kernel.  plain_persistent: 1 runs
 * the plain (no-HI) steps between two pair-list rebuilds as one launch with
 * one CTA per trajectory and the trajectory's frames in shared memory (for
 * batches whose largest trajectory has at most 2048 beads), 0 one launch
 * per step; both give identical results.
 * No reference counterpart (the reference launches everything with 32-thread
 * blocks, src/mt.h:34). */
typedef struct {
    int list_method;
    int step_block;
    int tea_slices;
    int tea_jparts;
    int plain_persistent;
} mtg_tuning;
int mtg_get_tuning(mtg_engine *e, mtg_tuning *t);
int mtg_set_tuning(mtg_engine *e, const mtg_tuning *t);
/* Times every candidate tuning over trial_steps steps from first_step
 * (CUDA events; each trial restarts from a snapshot of the state and noise
 * streams, which are restored afterwards, so the simulation is unchanged)
 * and keeps the fastest.  best / best_ms may be NULL. */
int mtg_autotune(mtg_engine *e, long long first_step, int trial_steps, mtg_tuning *best, float *best_ms);

/* ---- measurement ------------------------------------------------------- */
/* mtg_step bracketed by CUDA events recorded on the engine's stream;
 * *device_ms = the device time between them.  No reference counterpart (the
 * reference reports CPU clock() steps/s, src/timer.cpp:24-34). */
int mtg_step_timed(mtg_engine *e, long long first_step, int nsteps, float *device_ms);

/* Per-kernel timing: while enabled, every kernel launch of mtg_step is
 * bracketed by its own pair of CUDA events; after each mtg_step call the
 * durations of that call's launches are added to per-kind totals.  (When a
 * call replays a pair-list period graph more than once only its last replay
 * is counted; the call count below says how many launches were timed.)
 * Kinds: 0 pair-list rebuild, 1 fused plain step, 2 forces (+ TEA random
 * forces), 3 TEA epsilon pass, 4 TEA beta reduction, 5 TEA mobility step,
 * 6 learned-TEA descriptors + network + C_i/beta, 7 learned-TEA re-check,
 * 8 far-field proxies (charges and far potentials), 9 far-field near pairs,
 * 10 persistent run of plain steps (one launch covers the steps between two
 * pair-list rebuilds), 11 far-field interpolation + update.  With timing on,
 * the learned step's kernels run on one stream, one after another. */
#define MTG_KERNEL_KINDS 12
int mtg_set_kernel_timing(mtg_engine *e, int on);
int mtg_kernel_times(mtg_engine *e, double *total_ms, long long *launches, int reset);
/* Kernel launches replayed from the engine's step graphs since the last
 * reset: every kernel node of a captured list-period graph counts once per
 * replay (memset and event nodes do not).  Steps enqueued outside a graph
 * (ranges shorter than a period) are not counted here. */
int mtg_graph_kernel_launches(mtg_engine *e, long long *launches, int reset);

/* Measured FP32 FMA throughput of `device` in TFLOP/s: the best of
 * register-resident chains of scalar and of packed FP32x2 FMAs over 8 CTAs
 * per SM (5 runs each), the denominator of the roofline of the
 * FP32-pipe-bound TEA kernels. */
int mtg_measure_fp32_tflops(int device, double *tflops);

/* Architecture of the device code the library runs on `device`:
 * binary_version = 10 * major + minor of its SASS (103 for sm_103a),
 * ptx_version (may be NULL) of its PTX, from cudaFuncGetAttributes.  No
 * reference counterpart (a build check: the library carries sm_103a code). */
int mtg_device_code_version(int device, int *binary_version, int *ptx_version);

/* Page-locked host buffers for fast state transfers (cudaHostAlloc). */
int mtg_host_alloc(void **ptr, size_t bytes);
int mtg_host_free(void *ptr);

#ifdef __cplusplus
}
#endif

#endif /* MTG_H_ */
