// mtg_compute.cpp - drop-in replacement of the reference's compute() on top
// of the GB300 engine's C ABI.
//
// Build this file inside the reference project in place of
// src/compute_cuda.cu, src/bdhitea.cu, src/bdhitea_kernel.cu and
// src/HybridTaus.cu, and link mt_gb300/libmtg.so (see the Makefile next to
// this file).  It keeps the reference's signature
//     void compute(Coord* r, Coord* f, Parameters& par, Topology& top, Energies* energies)
// (src/compute_cuda.cuh:17, called from src/main.cpp:79), its host-side step
// loop order (src/compute_cuda.cu:1125-1260) and its updater hooks
// (update, mt_length, change_conc, hydrolyse from src/updater.cpp), while the
// device work goes through mtg_* calls.  A non-zero status becomes DIE(...),
// the reference's fatal-error behaviour (src/wrapper.h:22).
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "globals.h"
#include "mt.h"
#include "parameters.h"
#include "updater.h"
#include "wrapper.h"

#include "mtg.h"

namespace {

void check(int rc, const char *what) {
    if (rc != MTG_OK) DIE("%s failed (%d): %s", what, rc, mtg_last_error_string());
}

mtg_params to_mtg(const Parameters &par) {
    mtg_params p;
    std::memset(&p, 0, sizeof p);
    p.dt = par.dt;
    p.Temp = par.Temp;
    p.viscosity = par.viscosity;
    p.gammaR = par.gammaR;
    p.gammaTheta = par.gammaTheta;
    p.varR = par.varR;
    p.varTheta = par.varTheta;
    p.alpha = par.alpha;
    p.freeze_temp = par.freeze_temp;
    p.C = par.C;
    p.B_psi = par.B_psi;
    p.B_fi = par.B_fi;
    p.B_theta = par.B_theta;
    p.psi_0 = par.psi_0;
    p.fi_0 = par.fi_0;
    p.theta0_gtp = par.theta0_gtp;
    p.theta0_gdp = par.theta0_gdp;
    p.A_lat = par.A_lat;
    p.A_long = par.A_long;
    p.D_lat = par.D_lat;
    p.D_long = par.D_long;
    p.seam_coeff = par.seam_coeff;
    p.barrier = par.barrier;
    p.a_barr_long = par.a_barr_long;
    p.r_barr_long = par.r_barr_long;
    p.w_barr_long = par.w_barr_long;
    p.a_barr_lat = par.a_barr_lat;
    p.r_barr_lat = par.r_barr_lat;
    p.w_barr_lat = par.w_barr_lat;
    p.lj_on = par.lj_on;
    p.ljscale = par.ljscale;
    p.ljsigma6 = par.ljsigma6;
    p.ljpairscutoff = par.ljpairscutoff;
    p.ljpairsupdatefreq = par.ljpairsupdatefreq;
    p.is_wall = par.is_wall;
    p.rep_r = par.rep_r;
    p.rep_eps = par.rep_eps;
    p.rep_leftborder = par.rep_leftborder;
    p.is_assembly = par.is_assembly;
    p.hdi_on = par.hdi_on;
    p.tea_a = tea.a;
    p.tea_epsilon_freq = tea.epsilon_freq;
    p.tea_capricious = tea.capricious;
    p.tea_epsmax = tea.epsmax;
    p.rseed = par.rseed;
    p.device = par.device;
    return p;
}

}  // namespace

void compute(Coord *r, Coord *f, Parameters &par, Topology &top, Energies *energies) {
    const size_t nb = (size_t)par.Ntot * par.Ntr;
    // initIntegration's host part (src/compute_cuda.cu:995-1010): zero forces,
    // wrap angles once into (-2 pi, 2 pi)
    for (size_t i = 0; i < nb; i++) {
        f[i].x = f[i].y = f[i].z = f[i].fi = f[i].psi = f[i].theta = 0.0f;
        r[i].fi -= (2 * M_PI) * (int)(r[i].fi / (2 * M_PI));
        r[i].psi -= (2 * M_PI) * (int)(r[i].psi / (2 * M_PI));
        r[i].theta -= (2 * M_PI) * (int)(r[i].theta / (2 * M_PI));
    }
    mtg_params p = to_mtg(par);
    std::vector<uint8_t> fixed(par.Ntot), extra(nb);
    for (int i = 0; i < par.Ntot; i++) fixed[i] = top.fixed[i];
    for (size_t i = 0; i < nb; i++) extra[i] = top.extra[i];
    std::vector<float> zs(par.Ntr);
    for (int t = 0; t < par.Ntr; t++) zs[t] = par.zs[t];
    mtg_topology t;
    std::memset(&t, 0, sizeof t);
    t.Ntot = par.Ntot;
    t.Ntr = par.Ntr;
    t.maxHarmonicPerMonomer = top.maxHarmonicPerMonomer;
    t.harmonicCount = top.harmonicCount;
    t.harmonic = top.harmonic;
    t.maxLongitudinalPerMonomer = top.maxLongitudinalPerMonomer;
    t.longitudinalCount = top.longitudinalCount;
    t.longitudinal = top.longitudinal;
    t.maxLateralPerMonomer = top.maxLateralPerMonomer;
    t.lateralCount = top.lateralCount;
    t.lateral = top.lateral;
    t.maxLJPerMonomer = 256;  // src/compute_cuda.cu:1076
    t.fixed = fixed.data();
    t.mon_type = top.mon_type;
    t.extra = extra.data();
    t.gtp = top.gtp;
    t.on_tubule_cur = top.on_tubule_cur;
    t.zs = zs.data();

    mtg_engine *e = nullptr;
    check(mtg_create(&p, &t, &e), "mtg_create");
    check(mtg_upload_state(e, reinterpret_cast<const float *>(r)), "mtg_upload_state");

    std::vector<int> mt_len(par.Ntr, 0), mt_len_prev(par.Ntr, 0);
    const long long freq = par.ljpairsupdatefreq;
    long long step = 0;
    while (step < par.steps) {
        const bool hydro = par.hydrolysis && step % par.hydrostep == 0 && step != 0;
        const bool stride = step % par.stride == 0;
        if (hydro || stride) {
            // the reference rebuilds the lists before its host hooks (src/compute_cuda.cu:1140-1151)
            if (step % freq == 0) check(mtg_rebuild_pairs(e), "mtg_rebuild_pairs");
            if (hydro) {
                hydrolyse();
                check(mtg_set_gtp(e, top.gtp), "mtg_set_gtp");
            }
            if (stride) {
                if (par.out_energy) check(mtg_energies(e, reinterpret_cast<double *>(energies), nullptr), "mtg_energies");
                check(mtg_download_state(e, reinterpret_cast<float *>(r), par.out_force ? reinterpret_cast<float *>(f) : nullptr),
                      "mtg_download_state");
                if (par.out_force) {
                    // the reference's d_f holds no translational force here
                    // (zeroed by integrate_kernel / integrateTea_prepare), and no
                    // angular force either without TEA
                    for (size_t i = 0; i < nb; i++) {
                        f[i].x = f[i].y = f[i].z = 0.0f;
                        if (!par.hdi_on) f[i].fi = f[i].psi = f[i].theta = 0.0f;
                    }
                }
                if (par.tub_length) {
                    std::memcpy(top.on_tubule_prev, top.on_tubule_cur, nb * sizeof(int));
                    if (step != 0) {
                        mt_len_prev = mt_len;
                        mt_length(step, mt_len.data());
                        if (par.barrier) check(mtg_set_on_tubule(e, top.on_tubule_cur), "mtg_set_on_tubule");
                        if (par.is_const_conc) {
                            for (int i = 0; i < par.Ntr; i++) mt_len_prev[i] = mt_len[i] - mt_len_prev[i];
                            if (change_conc(mt_len_prev.data(), mt_len.data())) {
                                for (size_t i = 0; i < nb; i++) extra[i] = top.extra[i];
                                check(mtg_set_extra(e, extra.data()), "mtg_set_extra");
                                check(mtg_upload_state(e, reinterpret_cast<const float *>(r)), "mtg_upload_state");
                            }
                        }
                        update(step, mt_len.data());
                    } else {
                        update(step, mt_len.data());
                        mt_length(step, mt_len.data());
                    }
                } else {
                    update(step, mt_len.data());
                }
            }
            check(mtg_step(e, step, 1), "mtg_step");
            step++;
            continue;
        }
        // run to the next host event in one call (graph-replayed periods)
        long long next = par.steps;
        const long long ns = (step / par.stride + 1) * par.stride;
        if (ns < next) next = ns;
        if (par.hydrolysis) {
            const long long nh = (step / par.hydrostep + 1) * par.hydrostep;
            if (nh < next) next = nh;
        }
        check(mtg_step(e, step, (int)(next - step)), "mtg_step");
        step = next;
    }
    // deleteIntegration (src/compute_cuda.cu:1100-1123) copies nothing back:
    // on return r holds the state of the last stride step, which main() then
    // writes out (src/main.cpp:81)
    check(mtg_destroy(e), "mtg_destroy");
}
