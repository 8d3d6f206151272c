/*
 * mt_oracle.h - CPU oracle for the MADDY Brownian/Langevin hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * kernels (klyshko/MT src/compute_cuda.cu, src/bdhitea_kernel.cu,
 * src/bdhitea.cu, src/HybridTaus.cu, src/ran2.h) used by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg as the checker.
 * The product (mt_gb300/) never links or calls it.
 *
 * Parity of this oracle is pinned against the reference's own kernel bodies
 * compiled as host code (oracle/ref_harness.cpp -> oracle/_ref/libmtref.so,
 * built from the reference sources where they lie) and against the golden
 * fixtures under tests/golden/ that were generated from that build.
 *
 * Layout is the reference's: a uniform batch of Ntr trajectories x Ntot
 * beads, bead p = ind + traj*Ntot; Coord AoS of 7 REALs (x, y, z, fi, theta,
 * psi, w); lists bead-major with a fixed capacity per bead; HybridTaus
 * states as 4 uint32 per stream, 2*Ntot*Ntr streams.
 *
 * Every function exists twice: *_f32 computes in float (the reference's
 * arithmetic type) and *_f64 computes the same formulas in double (the error
 * yardstick).  The RNG integer stream is shared.
 */
#ifndef MT_ORACLE_H_
#define MT_ORACLE_H_

#include <stdint.h>
#include "../include/mtg.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ran2-based seeding of Np HybridTaus streams (src/HybridTaus.cu:32-48,
 * src/ran2.h:18-56); ran2's static state starts from its initial values. */
void orc_generate_seeds(int seed, int Np, uint32_t *seeds);
/* One HybridTaus draw (src/HybridTaus.cu:63-82) on state s[4]. */
uint32_t orc_hybrid_taus(uint32_t *s);
/* uintToFloat (src/HybridTaus.cu:53-61). */
float orc_uint_to_float(uint32_t u);
/* n successive rforce() calls on one stream (src/HybridTaus.cu:85-98):
 * out[4*k..4*k+3] = the k-th float4 of normals; the state advances. */
void orc_rforce_f32(uint32_t *s, int n, float *out);
void orc_rforce_f64(uint32_t *s, int n, double *out);

#define ORC_DECLARE(SUF, REAL)                                                                  \
    void orc_lj_list_##SUF(const mtg_params *p, const mtg_topology *t, const REAL *r,         \
                           int maxLJ, int *LJCount, int *LJ, int *overflow);                    \
    void orc_pairs_list_##SUF(const mtg_params *p, const mtg_topology *t, const REAL *r,      \
                              int maxLong, int *longCount, int *lon, int maxLat,                \
                              int *latCount, int *lat, int *overflow);                          \
    void orc_forces_##SUF(const mtg_params *p, const mtg_topology *t, const REAL *r,          \
                          int maxLong, const int *longCount, const int *lon, int maxLat,        \
                          const int *latCount, const int *lat, int maxLJ, const int *LJCount,   \
                          const int *LJ, REAL *f);                                              \
    void orc_energies_##SUF(const mtg_params *p, const mtg_topology *t, const REAL *r,        \
                            int maxLong, const int *longCount, const int *lon, int maxLat,      \
                            const int *latCount, const int *lat, int maxLJ,                     \
                            const int *LJCount, const int *LJ, double *en);                     \
    void orc_integrate_##SUF(const mtg_params *p, const mtg_topology *t, REAL *r, REAL *f,    \
                             uint32_t *seeds);                                                  \
    void orc_tea_prepare_##SUF(const mtg_params *p, const mtg_topology *t, REAL *f,           \
                               const REAL *r, uint32_t *seeds, REAL *rforce, REAL *mforce,      \
                               REAL *coords);                                                   \
    void orc_tea_epsilon_##SUF(const mtg_params *p, const mtg_topology *t, const REAL *r,     \
                               REAL *ci, REAL *eps);                                            \
    int orc_tea_beta_##SUF(const mtg_params *p, const mtg_topology *t, const REAL *eps,       \
                           double *eps_traj, REAL *beta);                                       \
    void orc_tea_integrate_##SUF(const mtg_params *p, const mtg_topology *t, REAL *f,         \
                                 REAL *r, uint32_t *seeds, const REAL *ci, const REAL *beta,    \
                                 const REAL *rforce, const REAL *mforce, const REAL *coords);   \
    int orc_run_##SUF(const mtg_params *p, const mtg_topology *t, REAL *r, REAL *f,           \
                      uint32_t *seeds, int maxLong, int *longCount, int *lon, int maxLat,       \
                      int *latCount, int *lat, int maxLJ, int *LJCount, int *LJ,                \
                      long long first_step, int nsteps, REAL *tea_ci, REAL *tea_beta);

ORC_DECLARE(f32, float)
ORC_DECLARE(f64, double)

#ifdef __cplusplus
}
#endif

#endif
