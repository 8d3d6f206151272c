// mtg_recorder.cpp - a recording stand-in for the engine's C ABI (test
// infrastructure).  Linked with mt_gb300/host/mtg_compute.cpp and the
// reference's own host program (main, preparator, updater, ...) instead of
// libmtg.so, it lets the drop-in compute() run on a CPU: every mtg_* call the
// drop-in makes is printed to stdout as one "MTG ..." line, in call order,
// between the reference program's own output lines.  The state is kept on
// the host unchanged (no dynamics), so the reference's hooks see the state
// the drop-in uploaded.  mtg_step logs the device work its contract promises
// (include/mtg.h): a pair-list rebuild at every step s with s %
// ljpairsupdatefreq == 0, except the first step of a call that follows
// mtg_rebuild_pairs, then the step itself.
//
// The reference's updater hooks are reached through the linker's --wrap:
// each __wrap_ function below prints one "HOOK ..." line and calls the
// reference's own function (__real_), so the order of hooks and engine calls
// is recorded exactly.
#include <cstdio>
#include <cstring>
#include <vector>

#include "mtg.h"

struct mtg_engine {
    mtg_params p;
    int nb, ntot, ntr;
    std::vector<float> state;
    bool fresh = false;
};

extern "C" {

const char *mtg_last_error_string(void) { return "recorder"; }

int mtg_create(const mtg_params *p, const mtg_topology *t, mtg_engine **out) {
    auto *e = new mtg_engine();
    e->p = *p;
    e->ntot = t->Ntot;
    e->ntr = t->Ntr;
    e->nb = t->Ntot * t->Ntr;
    e->state.assign((size_t)e->nb * MTG_COORD_FLOATS, 0.f);
    int nextra = 0;
    for (int i = 0; i < e->nb; i++) nextra += t->extra[i] ? 1 : 0;
    std::printf("MTG create Ntot=%d Ntr=%d maxH=%d maxLong=%d maxLat=%d maxLJ=%d extra=%d dt=%g Temp=%g "
                "viscosity=%g gammaR=%g gammaTheta=%g varR=%g varTheta=%g alpha=%g freeze_temp=%g C=%g B_psi=%g "
                "B_fi=%g B_theta=%g theta0_gdp=%g theta0_gtp=%g A_long=%g A_lat=%g D_long=%g D_lat=%g "
                "seam_coeff=%g barrier=%d lj_on=%d ljscale=%g ljpairscutoff=%g ljpairsupdatefreq=%d is_wall=%d "
                "rep_r=%g rep_eps=%g is_assembly=%d hdi_on=%d rseed=%d device=%d zs0=%g\n",
                t->Ntot, t->Ntr, t->maxHarmonicPerMonomer, t->maxLongitudinalPerMonomer, t->maxLateralPerMonomer,
                t->maxLJPerMonomer, nextra, p->dt, p->Temp, p->viscosity, p->gammaR, p->gammaTheta, p->varR,
                p->varTheta, p->alpha, p->freeze_temp, p->C, p->B_psi, p->B_fi, p->B_theta, p->theta0_gdp,
                p->theta0_gtp, p->A_long, p->A_lat, p->D_long, p->D_lat, p->seam_coeff, p->barrier, p->lj_on,
                p->ljscale, p->ljpairscutoff, p->ljpairsupdatefreq, p->is_wall, p->rep_r, p->rep_eps,
                p->is_assembly, p->hdi_on, p->rseed, p->device, t->zs ? t->zs[0] : -1.f);
    *out = e;
    return MTG_OK;
}

int mtg_destroy(mtg_engine *e) {
    std::printf("MTG destroy\n");
    delete e;
    return MTG_OK;
}

int mtg_upload_state(mtg_engine *e, const float *r) {
    std::memcpy(e->state.data(), r, e->state.size() * sizeof(float));
    double s = 0;
    for (float v : e->state) s += v;
    std::printf("MTG upload_state checksum=%.6e\n", s);
    return MTG_OK;
}

int mtg_download_state(mtg_engine *e, float *r, float *f) {
    if (r) std::memcpy(r, e->state.data(), e->state.size() * sizeof(float));
    // forces of the last step: none are kept by the stand-in
    if (f) std::memset(f, 0, e->state.size() * sizeof(float));
    std::printf("MTG download_state r=%d f=%d\n", r ? 1 : 0, f ? 1 : 0);
    return MTG_OK;
}

int mtg_rebuild_pairs(mtg_engine *e) {
    e->fresh = true;
    std::printf("MTG rebuild_pairs\n");
    return MTG_OK;
}

int mtg_set_gtp(mtg_engine *e, const int *gtp) {
    long n1 = 0;
    for (int i = 0; i < e->nb; i++) n1 += gtp[i] == 1;
    std::printf("MTG set_gtp gtp1=%ld\n", n1);
    return MTG_OK;
}

int mtg_set_extra(mtg_engine *e, const uint8_t *extra) {
    long n = 0;
    for (int i = 0; i < e->nb; i++) n += extra[i] != 0;
    std::printf("MTG set_extra extra=%ld\n", n);
    return MTG_OK;
}

int mtg_set_on_tubule(mtg_engine *e, const int *on) {
    long n = 0;
    for (int i = 0; i < e->nb; i++) n += on[i] != 0;
    std::printf("MTG set_on_tubule on=%ld\n", n);
    return MTG_OK;
}

int mtg_energies(mtg_engine *e, double *per_bead, double *per_traj) {
    if (per_bead) std::memset(per_bead, 0, sizeof(double) * MTG_ENERGY_TERMS * e->nb);
    if (per_traj) std::memset(per_traj, 0, sizeof(double) * MTG_ENERGY_TERMS * e->ntr);
    std::printf("MTG energies per_bead=%d per_traj=%d\n", per_bead ? 1 : 0, per_traj ? 1 : 0);
    return MTG_OK;
}

int mtg_step(mtg_engine *e, long long first, int n) {
    std::printf("MTG step_call first=%lld n=%d\n", first, n);
    const bool lists = e->p.lj_on || e->p.is_assembly;
    for (long long s = first; s < first + n; s++) {
        if (lists && s % e->p.ljpairsupdatefreq == 0 && !(s == first && e->fresh))
            std::printf("MTG device_rebuild step=%lld\n", s);
        std::printf("MTG device_step step=%lld\n", s);
    }
    if (n > 0) e->fresh = false;
    return MTG_OK;
}

}  // extern "C"

// ---- the reference's updater hooks (src/updater.h), wrapped ---------------
extern "C" {
void __real__Z9hydrolysev();
void __real__Z6updatexPi(long long, int *);
void __real__Z9mt_lengthxPi(long long, int *);
int __real__Z11change_concPiS_(int *, int *);

void __wrap__Z9hydrolysev() {
    std::printf("HOOK hydrolyse\n");
    __real__Z9hydrolysev();
}
void __wrap__Z6updatexPi(long long step, int *mt_len) {
    std::printf("HOOK update step=%lld\n", step);
    __real__Z6updatexPi(step, mt_len);
}
void __wrap__Z9mt_lengthxPi(long long step, int *mt_len) {
    std::printf("HOOK mt_length step=%lld\n", step);
    __real__Z9mt_lengthxPi(step, mt_len);
}
int __wrap__Z11change_concPiS_(int *delta, int *mt_len) {
    const int r = __real__Z11change_concPiS_(delta, mt_len);
    std::printf("HOOK change_conc ret=%d\n", r);
    return r;
}
}
