/*
 * ref_harness.cpp - drives the reference's own kernel bodies on the CPU.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/Makefile extracts, from the reference
 * tree, compute_cuda.cu:12-975 (kernels and __constant__ state),
 * HybridTaus.cu:1-20,31-98 (PRNG without the CUDA-only initRand) and
 * bdhitea_kernel.cu:16-213 (TEA kernels) into oracle/_ref/build/*.inc and
 * compiles them here with ref_shim.h, so that each "__global__" kernel is a
 * host function run once per bead.  The resulting oracle/_ref/libmtref.so
 * exposes the same entry points as the C oracle with a ref_ prefix (FP32
 * only); tests use it to pin the oracle and tests/golden/make_golden.py uses
 * it to write the golden fixtures.  Nothing of this file ships.
 *
 * The one piece restated here rather than executed is updateTea's host FP64
 * reduction (src/bdhitea.cu:57-118), which the reference interleaves with
 * cudaMemcpy calls.
 */
#include "compute_cuda.cuh"
#include "cc_part.inc"
#include "ht_part.inc"
#include "tea_part.inc"

#include <cstdint>
#include <cstring>
#include <vector>
#include "../include/mtg.h"

thread_local shim_dim3 blockIdx, threadIdx, blockDim;

namespace {

void set_params(const mtg_params *P, const mtg_topology *T) {
    Parameters par;
    std::memset(&par, 0, sizeof(par));
    par.hdi_on = P->hdi_on;
    par.rseed = P->rseed;
    par.Temp = P->Temp;
    par.varR = P->varR;
    par.gammaR = P->gammaR;
    par.varTheta = P->varTheta;
    par.gammaTheta = P->gammaTheta;
    par.viscosity = P->viscosity;
    par.freeze_temp = P->freeze_temp;
    par.is_assembly = P->is_assembly;
    par.alpha = P->alpha;
    par.dt = P->dt;
    par.Ntot = T->Ntot;
    par.Ntr = T->Ntr;
    par.C = P->C;
    par.B_psi = P->B_psi;
    par.B_fi = P->B_fi;
    par.B_theta = P->B_theta;
    par.psi_0 = P->psi_0;
    par.fi_0 = P->fi_0;
    par.theta0_gtp = P->theta0_gtp;
    par.theta0_gdp = P->theta0_gdp;
    par.A_lat = P->A_lat;
    par.A_long = P->A_long;
    par.D_lat = P->D_lat;
    par.D_long = P->D_long;
    par.seam_coeff = P->seam_coeff;
    par.is_wall = P->is_wall;
    par.rep_r = P->rep_r;
    par.rep_eps = P->rep_eps;
    par.rep_leftborder = P->rep_leftborder;
    for (int t = 0; t < T->Ntr && t < PARAMETER_LENGTH; t++) par.zs[t] = T->zs ? T->zs[t] : 0.f;
    par.barrier = P->barrier;
    par.a_barr_long = P->a_barr_long;
    par.r_barr_long = P->r_barr_long;
    par.w_barr_long = P->w_barr_long;
    par.a_barr_lat = P->a_barr_lat;
    par.r_barr_lat = P->r_barr_lat;
    par.w_barr_lat = P->w_barr_lat;
    par.ljpairscutoff = P->ljpairscutoff;
    par.ljpairsupdatefreq = P->ljpairsupdatefreq;
    par.lj_on = P->lj_on;
    par.ljscale = P->ljscale;
    par.ljsigma6 = P->ljsigma6;
    c_par = par;
}

void set_top(const mtg_topology *T, int maxLong, const int *longCount, const int *lon, int maxLat,
             const int *latCount, const int *lat, int maxLJ, const int *LJCount, const int *LJ) {
    Topology t;
    std::memset(&t, 0, sizeof(t));
    t.harmonicCount = const_cast<int *>(T->harmonicCount);
    t.harmonic = const_cast<int *>(T->harmonic);
    t.maxHarmonicPerMonomer = T->maxHarmonicPerMonomer;
    t.longitudinalCount = const_cast<int *>(longCount);
    t.longitudinal = const_cast<int *>(lon);
    t.maxLongitudinalPerMonomer = maxLong;
    t.lateralCount = const_cast<int *>(latCount);
    t.lateral = const_cast<int *>(lat);
    t.maxLateralPerMonomer = maxLat;
    t.LJCount = const_cast<int *>(LJCount);
    t.LJ = const_cast<int *>(LJ);
    t.maxLJPerMonomer = maxLJ;
    t.fixed = reinterpret_cast<bool *>(const_cast<uint8_t *>(T->fixed));
    t.extra = reinterpret_cast<bool *>(const_cast<uint8_t *>(T->extra));
    t.mon_type = const_cast<int *>(T->mon_type);
    t.gtp = const_cast<int *>(T->gtp);
    t.on_tubule_cur = const_cast<int *>(T->on_tubule_cur);
    t.on_tubule_prev = const_cast<int *>(T->on_tubule_cur);
    c_top = t;
}

template <class F>
void for_each_bead(int n, F &&kernel) {
    blockDim.x = 1;
    threadIdx.x = 0;
    for (int p = 0; p < n; p++) {
        blockIdx.x = (unsigned)p;
        kernel();
    }
}

}  // namespace

extern "C" {

void ref_generate_seeds(int seed, int Np, uint32_t *seeds) {
    generateSeeds(reinterpret_cast<uint4 *>(seeds), seed, Np);
}

void ref_rforce_f32(uint32_t *s, int n, float *out) {
    HybTau h = c_ht;
    h.d_seeds = reinterpret_cast<uint4 *>(s);
    c_ht = h;
    for (int k = 0; k < n; k++) {
        float4 v = rforce(0);
        out[4 * k + 0] = v.x;
        out[4 * k + 1] = v.y;
        out[4 * k + 2] = v.z;
        out[4 * k + 3] = v.w;
    }
}

void ref_forces_f32(const mtg_params *P, const mtg_topology *T, const float *r, int maxLong, const int *longCount,
                    const int *lon, int maxLat, const int *latCount, const int *lat, int maxLJ, const int *LJCount,
                    const int *LJ, float *f) {
    set_params(P, T);
    set_top(T, maxLong, longCount, lon, maxLat, latCount, lat, maxLJ, LJCount, LJ);
    for_each_bead(T->Ntot * T->Ntr, [&] {
        compute_kernel(reinterpret_cast<const Coord *>(r), reinterpret_cast<Coord *>(f));
    });
}

void ref_energies_f32(const mtg_params *P, const mtg_topology *T, const float *r, int maxLong, const int *longCount,
                      const int *lon, int maxLat, const int *latCount, const int *lat, int maxLJ, const int *LJCount,
                      const int *LJ, double *en) {
    set_params(P, T);
    set_top(T, maxLong, longCount, lon, maxLat, latCount, lat, maxLJ, LJCount, LJ);
    for_each_bead(T->Ntot * T->Ntr, [&] {
        energy_kernel(reinterpret_cast<const Coord *>(r), reinterpret_cast<Energies *>(en));
    });
}

void ref_lj_list_f32(const mtg_params *P, const mtg_topology *T, const float *r, int maxLJ, int *LJCount, int *LJ,
                     int *overflow) {
    (void)overflow;
    set_params(P, T);
    set_top(T, 0, nullptr, nullptr, 0, nullptr, nullptr, maxLJ, LJCount, LJ);
    for_each_bead(T->Ntot * T->Ntr, [&] { LJ_kernel(reinterpret_cast<const Coord *>(r)); });
}

void ref_pairs_list_f32(const mtg_params *P, const mtg_topology *T, const float *r, int maxLong, int *longCount,
                        int *lon, int maxLat, int *latCount, int *lat, int *overflow) {
    (void)overflow;
    set_params(P, T);
    set_top(T, maxLong, longCount, lon, maxLat, latCount, lat, 0, nullptr, nullptr);
    for_each_bead(T->Ntot * T->Ntr, [&] { pairs_kernel(reinterpret_cast<const Coord *>(r)); });
}

void ref_integrate_f32(const mtg_params *P, const mtg_topology *T, float *r, float *f, uint32_t *seeds) {
    set_params(P, T);
    set_top(T, 0, nullptr, nullptr, 0, nullptr, nullptr, 0, nullptr, nullptr);
    HybTau h = c_ht;
    h.d_seeds = reinterpret_cast<uint4 *>(seeds);
    c_ht = h;
    for_each_bead(T->Ntot * T->Ntr, [&] {
        integrate_kernel(reinterpret_cast<Coord *>(r), reinterpret_cast<Coord *>(f));
    });
}

static void set_tea(const mtg_params *P, const mtg_topology *T, float *rforce, float *mforce, float *coords,
                    float *ci, float *eps, float *beta) {
    Tea t;
    std::memset(&t, 0, sizeof(t));
    t.rforce = reinterpret_cast<float4 *>(rforce);
    t.mforce = reinterpret_cast<float4 *>(mforce);
    t.coords = reinterpret_cast<float4 *>(coords);
    t.d_ci = reinterpret_cast<float4 *>(ci);
    t.d_epsilon = eps;
    t.d_beta_ij = beta;
    t.epsilon_freq = P->tea_epsilon_freq;
    t.Ntot = T->Ntot;
    t.a = P->tea_a;
    t.capricious = P->tea_capricious;
    t.unlisted = 1;
    t.epsmax = P->tea_epsmax;
    c_tea = t;
}

void ref_tea_prepare_f32(const mtg_params *P, const mtg_topology *T, float *f, const float *r, uint32_t *seeds,
                         float *rforce, float *mforce, float *coords) {
    set_params(P, T);
    set_top(T, 0, nullptr, nullptr, 0, nullptr, nullptr, 0, nullptr, nullptr);
    set_tea(P, T, rforce, mforce, coords, nullptr, nullptr, nullptr);
    HybTau h = c_ht;
    h.d_seeds = reinterpret_cast<uint4 *>(seeds);
    c_ht = h;
    for_each_bead(T->Ntot * T->Ntr, [&] {
        integrateTea_prepare(reinterpret_cast<Coord *>(f), reinterpret_cast<Coord *>(const_cast<float *>(r)));
    });
}

void ref_tea_epsilon_f32(const mtg_params *P, const mtg_topology *T, const float *r, float *ci, float *eps) {
    set_params(P, T);
    set_top(T, 0, nullptr, nullptr, 0, nullptr, nullptr, 0, nullptr, nullptr);
    set_tea(P, T, nullptr, nullptr, nullptr, ci, eps, nullptr);
    for_each_bead(T->Ntot * T->Ntr, [&] {
        integrateTea_epsilon_unlisted(reinterpret_cast<Coord *>(const_cast<float *>(r)));
    });
}

void ref_tea_integrate_f32(const mtg_params *P, const mtg_topology *T, float *f, float *r, uint32_t *seeds,
                           const float *ci, const float *beta, const float *rforce, const float *mforce,
                           const float *coords) {
    set_params(P, T);
    set_top(T, 0, nullptr, nullptr, 0, nullptr, nullptr, 0, nullptr, nullptr);
    set_tea(P, T, const_cast<float *>(rforce), const_cast<float *>(mforce), const_cast<float *>(coords),
            const_cast<float *>(ci), nullptr, const_cast<float *>(beta));
    HybTau h = c_ht;
    h.d_seeds = reinterpret_cast<uint4 *>(seeds);
    c_ht = h;
    for_each_bead(T->Ntot * T->Ntr, [&] {
        integrateTea_kernel_unlisted(reinterpret_cast<Coord *>(f), reinterpret_cast<Coord *>(r));
    });
}

}  // extern "C"
