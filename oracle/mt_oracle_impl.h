/*
 * mt_oracle_impl.h - body of the CPU oracle, included by mt_oracle.c once per
 * precision with REAL, SUF, MSQRT/MSIN/MCOS/MEXP/MLOG/MFABS defined.
 *
 * TEST INFRASTRUCTURE ONLY (see mt_oracle.h).
 *
 * The orientation of a bead is the rotation R = Rz(psi) Ry(theta) Rx(fi);
 * a binding site s (body frame) sits at r + R s.  The reference writes the
 * site-to-site vectors and their angular gradients out term by term
 * (src/compute_cuda.cu:86-129 harmonic, :205-247 longitudinal, :333-437
 * lateral); here the same quantities come from R and from the identity
 * d/d(angle) (R s) = axis x (R s), axis = z (psi), Rz(psi) y (theta),
 * R x (fi), which gives the generalised forces as projections of the torque
 * sum_pairs dU/dr / r * (R s) x d.
 */

#define CAT2(a, b) a##_##b
#define CAT(a, b) CAT2(a, b)
#define FN(name) CAT(name, SUF)

typedef struct {
    REAL x, y, z;
} CAT(vec3, SUF);
#define V3 CAT(vec3, SUF)

/* Binding-site geometry of the reference (src/mt.h:23-50): r_mon = 2 nm,
 * R_MT = 8.12 nm, lateral sites p1/p2, longitudinal site at +-r_mon along the
 * bead's z axis, ANGLE_CUTOFF 1 nm, PAIR_CUTOFF 2.5 nm, LJ force cutoff 6 nm. */
static void FN(lateral_sites)(V3 *p1, V3 *p2) {
    const REAL rmt = (REAL)8.12f, rmon = (REAL)2.0f;
    const REAL c = MCOS((REAL)(2.0 * M_PI / 13.0)), s = MSIN((REAL)(2.0 * M_PI / 13.0));
    p1->x = (REAL)0.5 * rmt * (c - (REAL)1);
    p1->y = (REAL)0.5 * rmt * s;
    p1->z = (REAL)-3 * rmon / (REAL)13;
    p2->x = p1->x;
    p2->y = -p1->y;
    p2->z = -p1->z;
}

typedef struct {
    REAL m[3][3];      /* rotation matrix */
    V3 ax_psi, ax_theta, ax_fi;
} CAT(frame, SUF);
#define FRAME CAT(frame, SUF)

static void FN(make_frame)(REAL fi, REAL theta, REAL psi, FRAME *F) {
    const REAL sf = MSIN(fi), cf = MCOS(fi), st = MSIN(theta), ct = MCOS(theta);
    const REAL sp = MSIN(psi), cp = MCOS(psi);
    F->m[0][0] = cp * ct;
    F->m[0][1] = cp * st * sf - sp * cf;
    F->m[0][2] = cp * st * cf + sp * sf;
    F->m[1][0] = sp * ct;
    F->m[1][1] = sp * st * sf + cp * cf;
    F->m[1][2] = sp * st * cf - cp * sf;
    F->m[2][0] = -st;
    F->m[2][1] = ct * sf;
    F->m[2][2] = ct * cf;
    F->ax_psi.x = 0; F->ax_psi.y = 0; F->ax_psi.z = 1;
    F->ax_theta.x = -sp; F->ax_theta.y = cp; F->ax_theta.z = 0;
    F->ax_fi.x = F->m[0][0]; F->ax_fi.y = F->m[1][0]; F->ax_fi.z = F->m[2][0];
}

static V3 FN(rot)(const FRAME *F, V3 s) {
    V3 o;
    o.x = F->m[0][0] * s.x + F->m[0][1] * s.y + F->m[0][2] * s.z;
    o.y = F->m[1][0] * s.x + F->m[1][1] * s.y + F->m[1][2] * s.z;
    o.z = F->m[2][0] * s.x + F->m[2][1] * s.y + F->m[2][2] * s.z;
    return o;
}

/* coordinate accessors for Coord AoS (x, y, z, fi, theta, psi, w) */
#define CX(r, p) (r)[7 * (size_t)(p) + 0]
#define CY(r, p) (r)[7 * (size_t)(p) + 1]
#define CZ(r, p) (r)[7 * (size_t)(p) + 2]
#define CFI(r, p) (r)[7 * (size_t)(p) + 3]
#define CTH(r, p) (r)[7 * (size_t)(p) + 4]
#define CPS(r, p) (r)[7 * (size_t)(p) + 5]

static FRAME FN(bead_frame)(const REAL *r, size_t p) {
    FRAME F;
    FN(make_frame)(CFI(r, p), CTH(r, p), CPS(r, p), &F);
    return F;
}

/* d = (r_j + w_j) - (r_i + w_i); position difference first */
static V3 FN(site_delta)(const REAL *r, size_t pi, size_t pj, V3 wi, V3 wj) {
    V3 d;
    d.x = ((CX(r, pj) - CX(r, pi)) + wj.x) - wi.x;
    d.y = ((CY(r, pj) - CY(r, pi)) + wj.y) - wi.y;
    d.z = ((CZ(r, pj) - CZ(r, pi)) + wj.z) - wi.z;
    return d;
}

static REAL FN(norm)(V3 d) { return MSQRT(d.x * d.x + d.y * d.y + d.z * d.z); }

static V3 FN(scale)(V3 a, REAL s) {
    a.x *= s; a.y *= s; a.z *= s;
    return a;
}

/* Morse derivative and energy, Gaussian barrier (src/compute_cuda.cu:16-30) */
static REAL FN(dmorse)(REAL D, REAL a, REAL x) {
    const REAL e = MEXP(-a * x);
    return 2 * a * D * (1 - e) * e;
}
static REAL FN(morse_en)(REAL D, REAL a, REAL x) {
    const REAL e = MEXP(-a * x);
    return D * (1 - e) * (1 - e) - D;
}
static REAL FN(dbarr)(REAL a, REAL r0, REAL w, REAL x) {
    return -a * MEXP(-(x - r0) * (x - r0) / (2 * w * w)) * (x - r0) / (w * w);
}
static REAL FN(barr)(REAL a, REAL r0, REAL w, REAL x) {
    return a * MEXP(-(x - r0) * (x - r0) / (2 * w * w));
}

/* Accumulators of one bead's generalised force. */
typedef struct {
    REAL fx, fy, fz, ffi, fpsi, ftheta;
    REAL tx, ty, tz; /* torque-like sum of dUdr * (w_i x d) */
} CAT(acc, SUF);
#define ACC CAT(acc, SUF)

static void FN(acc_pair)(ACC *A, REAL dUdr, V3 d, V3 wi) {
    A->fx += dUdr * d.x;
    A->fy += dUdr * d.y;
    A->fz += dUdr * d.z;
    A->tx += dUdr * (wi.y * d.z - wi.z * d.y);
    A->ty += dUdr * (wi.z * d.x - wi.x * d.z);
    A->tz += dUdr * (wi.x * d.y - wi.y * d.x);
}

static REAL FN(dot)(V3 a, REAL x, REAL y, REAL z) { return a.x * x + a.y * y + a.z * z; }

/* Decoding of a longitudinal/harmonic entry: j < 0 -> R_MON = +r_mon
 * (src/compute_cuda.cu:72-78). */
static int FN(decode_axial)(int e, REAL *rmon) {
    if (e < 0) {
        *rmon = (REAL)2.0f;
        return -e;
    }
    *rmon = (REAL)-2.0f;
    return e;
}
/* Decoding of a lateral entry: j <= 0 selects (i: p1, j: p2), otherwise
 * (i: p2, j: p1); +-ZERO (999999) encodes bead 0 (src/compute_cuda.cu:307-324). */
static int FN(decode_lateral)(int e, int *neg) {
    *neg = (e <= 0);
    int j = e < 0 ? -e : e;
    if (j == 999999) j = 0;
    return j;
}

/* ---------------------------------------------------------------- forces */
/* compute_kernel (src/compute_cuda.cu:32-525), one bead at a time. */
void FN(orc_forces)(const mtg_params *P, const mtg_topology *T, const REAL *r, int maxLong,
                    const int *longCount, const int *lon, int maxLat, const int *latCount,
                    const int *lat, int maxLJ, const int *LJCount, const int *LJ, REAL *f) {
    const int N = T->Ntot, Ntr = T->Ntr;
    V3 P1, P2;
    FN(lateral_sites)(&P1, &P2);
    const REAL lj_pref = (REAL)P->ljscale * (REAL)P->ljsigma6;
    const long long NN = (long long)N * Ntr;
    ORC_PAR_FOR
    for (long long pp = 0; pp < NN; pp++) {
        {
            const size_t p = (size_t)pp;
            const int traj = (int)(pp / N), ind = (int)(pp % N);
            if (T->extra[p]) continue; /* d_f[p] left untouched (:55) */
            ACC A = {0, 0, 0, 0, 0, 0, 0, 0, 0};
            const FRAME Fi = FN(bead_frame)(r, p);
            const V3 ez = {0, 0, 1};
            const V3 uzi = FN(rot)(&Fi, ez);
            /* harmonic bond within the dimer + bending (:69-182) */
            for (int k = 0; k < T->harmonicCount[ind]; k++) {
                REAL rmon;
                const int j = FN(decode_axial)(T->harmonic[T->maxHarmonicPerMonomer * ind + k], &rmon);
                const size_t pj = (size_t)j + (size_t)traj * N;
                const FRAME Fj = FN(bead_frame)(r, pj);
                const V3 wi = FN(scale)(uzi, rmon);
                const V3 wj = FN(scale)(FN(rot)(&Fj, ez), -rmon);
                const V3 d = FN(site_delta)(r, p, pj, wi, wj);
                const REAL dr = FN(norm)(d);
                FN(acc_pair)(&A, (REAL)P->C, d, wi);
                if (dr < (REAL)1.0f) {
                    const REAL th0 = T->gtp[p] == 1 ? (REAL)P->theta0_gtp : (REAL)P->theta0_gdp;
                    const REAL dpsi = CPS(r, pj) - CPS(r, p), dfi = CFI(r, pj) - CFI(r, p);
                    const REAL dth = CTH(r, pj) - CTH(r, p);
                    if (rmon > 0) {
                        A.fpsi += (REAL)P->B_psi * MSIN(dpsi - (REAL)P->psi_0);
                        A.ffi += (REAL)P->B_fi * MSIN(dfi - (REAL)P->fi_0);
                        A.ftheta += (REAL)P->B_theta * MSIN(dth - th0);
                    } else {
                        A.fpsi -= (REAL)P->B_psi * MSIN(-dpsi - (REAL)P->psi_0);
                        A.ffi -= (REAL)P->B_fi * MSIN(-dfi - (REAL)P->fi_0);
                        A.ftheta -= (REAL)P->B_theta * MSIN(-dth - th0);
                    }
                }
            }
            /* Morse longitudinal + bending (:187-301) */
            for (int k = 0; k < longCount[p]; k++) {
                REAL rmon;
                const int j = FN(decode_axial)(lon[(size_t)maxLong * p + k], &rmon);
                const size_t pj = (size_t)j + (size_t)traj * N;
                const FRAME Fj = FN(bead_frame)(r, pj);
                const V3 wi = FN(scale)(uzi, rmon);
                const V3 wj = FN(scale)(FN(rot)(&Fj, ez), -rmon);
                const V3 d = FN(site_delta)(r, p, pj, wi, wj);
                const REAL dr = FN(norm)(d);
                REAL dUdr = dr == 0 ? (REAL)0 : FN(dmorse)((REAL)P->D_long, (REAL)P->A_long, dr) / dr;
                if (P->barrier && T->on_tubule_cur[p] == 0 && T->on_tubule_cur[pj] == 0 && dr != 0)
                    dUdr += FN(dbarr)((REAL)P->a_barr_long, (REAL)P->r_barr_long, (REAL)P->w_barr_long, dr) / dr;
                FN(acc_pair)(&A, dUdr, d, wi);
                if (dr < (REAL)1.0f) {
                    /* theta0 of the bead nearer the plus end (:282-283) */
                    const size_t last = CZ(r, p) > CZ(r, pj) ? p : pj;
                    const REAL th0 = T->gtp[last] == 1 ? (REAL)P->theta0_gtp : (REAL)P->theta0_gdp;
                    const REAL dpsi = CPS(r, pj) - CPS(r, p), dfi = CFI(r, pj) - CFI(r, p);
                    const REAL dth = CTH(r, pj) - CTH(r, p);
                    if (rmon > 0) {
                        A.fpsi += (REAL)P->B_psi * MSIN(dpsi - (REAL)P->psi_0);
                        A.ffi += (REAL)P->B_fi * MSIN(dfi - (REAL)P->fi_0);
                        A.ftheta += (REAL)P->B_theta * MSIN(dth - th0);
                    } else {
                        A.fpsi -= (REAL)P->B_psi * MSIN(-dpsi - (REAL)P->psi_0);
                        A.ffi -= (REAL)P->B_fi * MSIN(-dfi - (REAL)P->fi_0);
                        A.ftheta -= (REAL)P->B_theta * MSIN(-dth - th0);
                    }
                }
            }
            /* Morse lateral with seam coefficient (:303-467) */
            for (int k = 0; k < latCount[p]; k++) {
                int neg;
                const int j = FN(decode_lateral)(lat[(size_t)maxLat * p + k], &neg);
                const size_t pj = (size_t)j + (size_t)traj * N;
                const FRAME Fj = FN(bead_frame)(r, pj);
                const V3 wi = FN(rot)(&Fi, neg ? P1 : P2);
                const V3 wj = FN(rot)(&Fj, neg ? P2 : P1);
                const V3 d = FN(site_delta)(r, p, pj, wi, wj);
                const REAL dr = FN(norm)(d);
                REAL dUdr;
                if (dr == 0)
                    dUdr = 0;
                else if (T->mon_type[ind] != T->mon_type[j])
                    dUdr = FN(dmorse)((REAL)P->D_lat / (REAL)P->seam_coeff, (REAL)P->A_lat, dr) / dr;
                else
                    dUdr = FN(dmorse)((REAL)P->D_lat, (REAL)P->A_lat, dr) / dr;
                if (P->barrier && T->on_tubule_cur[p] == 0 && T->on_tubule_cur[pj] == 0 && dr != 0)
                    dUdr += FN(dbarr)((REAL)P->a_barr_lat, (REAL)P->r_barr_lat, (REAL)P->w_barr_lat, dr) / dr;
                FN(acc_pair)(&A, dUdr, d, wi);
            }
            /* LJ r^-6 repulsion inside the hard 6 nm cutoff (:470-495) */
            if (P->lj_on) {
                for (int k = 0; k < LJCount[p]; k++) {
                    const size_t pj = (size_t)LJ[(size_t)maxLJ * p + k] + (size_t)traj * N;
                    const REAL dx = CX(r, p) - CX(r, pj), dy = CY(r, p) - CY(r, pj), dz = CZ(r, p) - CZ(r, pj);
                    const REAL dr = MSQRT(dx * dx + dy * dy + dz * dz);
                    if (dr < (REAL)6.0) {
                        const REAL dr2 = dr * dr, dr4 = dr2 * dr2;
                        const REAL df = (REAL)6 / (dr4 * dr4);
                        A.fx += lj_pref * df * dx;
                        A.fy += lj_pref * df * dy;
                        A.fz += lj_pref * df * dz;
                    }
                }
            }
            /* cylindrical walls (:497-517) */
            if (P->is_wall) {
                const REAL z = CZ(r, p), lb = (REAL)P->rep_leftborder;
                const REAL top = (REAL)T->zs[traj] + lb;
                if (z < lb)
                    A.fz += (REAL)P->rep_eps * MFABS(z - lb);
                else if (z > top)
                    A.fz += -(REAL)P->rep_eps * MFABS(z - top);
                const REAL rad2 = CX(r, p) * CX(r, p) + CY(r, p) * CY(r, p);
                if (rad2 > (REAL)P->rep_r * (REAL)P->rep_r) {
                    const REAL rad = MSQRT(rad2);
                    const REAL coeff = -(REAL)P->rep_eps * (rad - (REAL)P->rep_r);
                    A.fx += CX(r, p) / rad * coeff;
                    A.fy += CY(r, p) / rad * coeff;
                }
            }
            REAL *fo = f + 7 * p;
            fo[0] = A.fx;
            fo[1] = A.fy;
            fo[2] = A.fz;
            fo[3] = A.ffi + FN(dot)(Fi.ax_fi, A.tx, A.ty, A.tz);
            fo[4] = A.ftheta + FN(dot)(Fi.ax_theta, A.tx, A.ty, A.tz);
            fo[5] = A.fpsi + FN(dot)(Fi.ax_psi, A.tx, A.ty, A.tz);
            fo[6] = 0;
        }
    }
}

/* -------------------------------------------------------------- energies */
/* energy_kernel (src/compute_cuda.cu:676-911): per-bead terms accumulated in
 * REAL and halved; en[7*p + term], terms in Energies order. */
void FN(orc_energies)(const mtg_params *P, const mtg_topology *T, const REAL *r, int maxLong,
                      const int *longCount, const int *lon, int maxLat, const int *latCount,
                      const int *lat, int maxLJ, const int *LJCount, const int *LJ, double *en) {
    const int N = T->Ntot, Ntr = T->Ntr;
    V3 P1, P2;
    FN(lateral_sites)(&P1, &P2);
    const long long NN = (long long)N * Ntr;
    ORC_PAR_FOR
    for (long long pp = 0; pp < NN; pp++) {
        {
            const size_t p = (size_t)pp;
            const int traj = (int)(pp / N), ind = (int)(pp % N);
            REAL Uh = 0, Ulong = 0, Ulat = 0, Upsi = 0, Ufi = 0, Uth = 0, Ulj = 0;
            if (!T->extra[p]) {
                const FRAME Fi = FN(bead_frame)(r, p);
                const V3 ez = {0, 0, 1};
                const V3 uzi = FN(rot)(&Fi, ez);
                for (int k = 0; k < T->harmonicCount[ind]; k++) {
                    REAL rmon;
                    const int j = FN(decode_axial)(T->harmonic[T->maxHarmonicPerMonomer * ind + k], &rmon);
                    const size_t pj = (size_t)j + (size_t)traj * N;
                    const FRAME Fj = FN(bead_frame)(r, pj);
                    const V3 d = FN(site_delta)(r, p, pj, FN(scale)(uzi, rmon), FN(scale)(FN(rot)(&Fj, ez), -rmon));
                    const REAL dr = FN(norm)(d);
                    Uh += ((REAL)P->C / 2) * dr * dr;
                    if (dr < (REAL)1.0f) {
                        /* psi_ij, fi_ij and theta_ji (Q6 of the reference, :751-756) */
                        const REAL th0 = T->gtp[p] == 1 ? (REAL)P->theta0_gtp : (REAL)P->theta0_gdp;
                        Upsi += (REAL)P->B_psi * (1 - MCOS((CPS(r, p) - CPS(r, pj)) - (REAL)P->psi_0));
                        Ufi += (REAL)P->B_fi * (1 - MCOS((CFI(r, p) - CFI(r, pj)) - (REAL)P->fi_0));
                        Uth += (REAL)P->B_theta * (1 - MCOS((CTH(r, pj) - CTH(r, p)) - th0));
                    }
                }
                for (int k = 0; k < longCount[p]; k++) {
                    REAL rmon;
                    const int j = FN(decode_axial)(lon[(size_t)maxLong * p + k], &rmon);
                    const size_t pj = (size_t)j + (size_t)traj * N;
                    const FRAME Fj = FN(bead_frame)(r, pj);
                    const V3 d = FN(site_delta)(r, p, pj, FN(scale)(uzi, rmon), FN(scale)(FN(rot)(&Fj, ez), -rmon));
                    const REAL dr = FN(norm)(d);
                    Ulong += FN(morse_en)((REAL)P->D_long, (REAL)P->A_long, dr);
                    if (P->barrier && T->on_tubule_cur[p] == 0 && T->on_tubule_cur[pj] == 0)
                        Ulong += FN(barr)((REAL)P->a_barr_long, (REAL)P->r_barr_long, (REAL)P->w_barr_long, dr);
                    if (dr < (REAL)1.0f) {
                        const size_t last = CZ(r, p) > CZ(r, pj) ? p : pj;
                        const REAL th0 = T->gtp[last] == 1 ? (REAL)P->theta0_gtp : (REAL)P->theta0_gdp;
                        Upsi += (REAL)P->B_psi * (1 - MCOS((CPS(r, p) - CPS(r, pj)) - (REAL)P->psi_0));
                        Ufi += (REAL)P->B_fi * (1 - MCOS((CFI(r, p) - CFI(r, pj)) - (REAL)P->fi_0));
                        Uth += (REAL)P->B_theta * (1 - MCOS((CTH(r, p) - CTH(r, pj)) - th0));
                    }
                }
                for (int k = 0; k < latCount[p]; k++) {
                    int neg;
                    const int j = FN(decode_lateral)(lat[(size_t)maxLat * p + k], &neg);
                    const size_t pj = (size_t)j + (size_t)traj * N;
                    const FRAME Fj = FN(bead_frame)(r, pj);
                    const V3 d = FN(site_delta)(r, p, pj, FN(rot)(&Fi, neg ? P1 : P2), FN(rot)(&Fj, neg ? P2 : P1));
                    const REAL dr = FN(norm)(d);
                    if (T->mon_type[ind] != T->mon_type[j])
                        Ulat += FN(morse_en)((REAL)P->D_lat / (REAL)P->seam_coeff, (REAL)P->A_lat, dr);
                    else
                        Ulat += FN(morse_en)((REAL)P->D_lat, (REAL)P->A_lat, dr);
                    if (P->barrier && T->on_tubule_cur[p] == 0 && T->on_tubule_cur[pj] == 0)
                        Ulat += FN(barr)((REAL)P->a_barr_lat, (REAL)P->r_barr_lat, (REAL)P->w_barr_lat, dr);
                }
                if (P->lj_on) {
                    for (int k = 0; k < LJCount[p]; k++) {
                        const size_t pj = (size_t)LJ[(size_t)maxLJ * p + k] + (size_t)traj * N;
                        const REAL dx = CX(r, p) - CX(r, pj), dy = CY(r, p) - CY(r, pj), dz = CZ(r, p) - CZ(r, pj);
                        const REAL dr2 = dx * dx + dy * dy + dz * dz;
                        const REAL dr = MSQRT(dr2);
                        if (dr < (REAL)6.0) Ulj += (REAL)P->ljscale * (REAL)P->ljsigma6 / (dr2 * dr2 * dr2);
                    }
                }
            }
            double *e = en + 7 * p;
            e[0] = (double)(Uh / 2);
            e[1] = (double)(Ulong / 2);
            e[2] = (double)(Ulat / 2);
            e[3] = (double)(Upsi / 2);
            e[4] = (double)(Ufi / 2);
            e[5] = (double)(Uth / 2);
            e[6] = (double)(Ulj / 2);
        }
    }
}

/* ------------------------------------------------------------- pair lists */
/* Distance between two bead centres, fixed FP32-reproducible order:
 * ((dx*dx + dy*dy) + dz*dz), then sqrt. */
static REAL FN(centre_dist)(const REAL *r, size_t a, size_t b) {
    const REAL dx = CX(r, a) - CX(r, b), dy = CY(r, a) - CY(r, b), dz = CZ(r, a) - CZ(r, b);
    const REAL dx2 = dx * dx, dy2 = dy * dy, dz2 = dz * dz;
    return MSQRT((dx2 + dy2) + dz2);
}

/* LJ_kernel (src/compute_cuda.cu:913-940): j != i within ljpairscutoff, in
 * ascending j, extra j included, empty list for an extra i.  Entries past
 * maxLJ are dropped and flagged (the reference writes past the end). */
void FN(orc_lj_list)(const mtg_params *P, const mtg_topology *T, const REAL *r, int maxLJ,
                     int *LJCount, int *LJ, int *overflow) {
    const int N = T->Ntot, Ntr = T->Ntr;
    const REAL cut = (REAL)P->ljpairscutoff;
    const long long NN = (long long)N * Ntr;
    ORC_PAR_FOR
    for (long long pp = 0; pp < NN; pp++) {
        {
            const size_t p = (size_t)pp;
            const int tr = (int)(pp / N), i = (int)(pp % N);
            int cnt = 0;
            if (!T->extra[p]) {
                for (int j = 0; j < N; j++) {
                    const size_t pj = (size_t)j + (size_t)tr * N;
                    if (i != j && FN(centre_dist)(r, p, pj) < cut) {
                        if (cnt < maxLJ)
                            LJ[(size_t)maxLJ * p + cnt] = j;
                        else if (overflow)
                            ORC_SET_FLAG(*overflow);
                        cnt++;
                    }
                }
            }
            LJCount[p] = cnt < maxLJ ? cnt : maxLJ;
        }
    }
}

/* pairs_kernel (src/compute_cuda.cu:527-674), assembly mode. */
void FN(orc_pairs_list)(const mtg_params *P, const mtg_topology *T, const REAL *r, int maxLong,
                        int *longCount, int *lon, int maxLat, int *latCount, int *lat, int *overflow) {
    (void)P;
    const int N = T->Ntot, Ntr = T->Ntr;
    V3 P1, P2;
    FN(lateral_sites)(&P1, &P2);
    const V3 ez = {0, 0, 1};
    const REAL cut = (REAL)2.5f;
    const long long NN = (long long)N * Ntr;
    ORC_PAR_FOR
    for (long long pp = 0; pp < NN; pp++) {
        {
            const size_t p = (size_t)pp;
            const int tr = (int)(pp / N), i = (int)(pp % N);
            int nl = 0, nt = 0;
            if (!T->extra[p]) {
                /* harmonic[max*i] < 0 (partner above, or no partner: -1) -> R_MON = -r_mon */
                const int h0 = T->harmonic[T->maxHarmonicPerMonomer * i];
                const REAL rmon = h0 < 0 ? (REAL)-2.0f : (REAL)2.0f;
                const int hpart = h0 < 0 ? -h0 : h0;
                const FRAME Fi = FN(bead_frame)(r, p);
                const V3 wi = FN(scale)(FN(rot)(&Fi, ez), rmon);
                const V3 li1 = FN(rot)(&Fi, P1), li2 = FN(rot)(&Fi, P2);
                for (int j = 0; j < N; j++) {
                    if (T->mon_type[i] == T->mon_type[j] || hpart == j) continue;
                    const size_t pj = (size_t)j + (size_t)tr * N;
                    const FRAME Fj = FN(bead_frame)(r, pj);
                    const V3 d = FN(site_delta)(r, p, pj, wi, FN(scale)(FN(rot)(&Fj, ez), -rmon));
                    if (FN(norm)(d) < cut) {
                        if (nl < maxLong)
                            lon[(size_t)maxLong * p + nl] = h0 < 0 ? j : -j;
                        else if (overflow)
                            ORC_SET_FLAG(*overflow);
                        nl++;
                    }
                }
                for (int j = 0; j < N; j++) {
                    if (i == j || hpart == j) continue;
                    const size_t pj = (size_t)j + (size_t)tr * N;
                    const FRAME Fj = FN(bead_frame)(r, pj);
                    const V3 lj1 = FN(rot)(&Fj, P1), lj2 = FN(rot)(&Fj, P2);
                    for (int o = 0; o < 2; o++) {
                        /* o = 0: i site p1, j site p2 -> -j; o = 1: i site p2, j site p1 -> +j */
                        const V3 d = FN(site_delta)(r, p, pj, o == 0 ? li1 : li2, o == 0 ? lj2 : lj1);
                        if (FN(norm)(d) < cut) {
                            const int code = j != 0 ? j : 999999;
                            if (nt < maxLat)
                                lat[(size_t)maxLat * p + nt] = o == 0 ? -code : code;
                            else if (overflow)
                                ORC_SET_FLAG(*overflow);
                            nt++;
                        }
                    }
                }
            }
            longCount[p] = nl < maxLong ? nl : maxLong;
            latCount[p] = nt < maxLat ? nt : maxLat;
        }
    }
}

/* -------------------------------------------------------------------- RNG */
void FN(orc_rforce)(uint32_t *s, int n, REAL *out) {
    for (int k = 0; k < n; k++) {
        for (int h = 0; h < 2; h++) {
            const float u1 = orc_uint_to_float(orc_hybrid_taus(s));
            const float u2 = orc_uint_to_float(orc_hybrid_taus(s));
            const REAL rad = MSQRT((REAL)-2.0 * MLOG((REAL)u1));
            const REAL th = (REAL)(2.0f * M_PI * u2);
            out[4 * k + 2 * h + 0] = rad * MSIN(th);
            out[4 * k + 2 * h + 1] = rad * MCOS(th);
        }
    }
}

/* --------------------------------------------------------------- integrate */
/* integrate_kernel (src/compute_cuda.cu:943-975): EM update of moving beads,
 * consuming streams p (xyz) and p + Ntot*Ntr (angles); forces zeroed. */
void FN(orc_integrate)(const mtg_params *P, const mtg_topology *T, REAL *r, REAL *f, uint32_t *seeds) {
    const size_t NN = (size_t)T->Ntot * T->Ntr;
    const REAL kr = (REAL)P->dt / (REAL)P->gammaR;
    const REAL kfi = (REAL)P->dt / ((REAL)P->gammaTheta * (REAL)P->alpha);
    const REAL kth = (REAL)P->dt / (REAL)P->gammaTheta;
    const REAL nfi = (REAL)P->varTheta * MSQRT((REAL)P->freeze_temp / (REAL)P->alpha);
    ORC_PAR_FOR
    for (size_t p = 0; p < NN; p++) {
        if (!T->fixed[p % T->Ntot] && !T->extra[p]) {
            REAL a[4], b[4];
            FN(orc_rforce)(seeds + 4 * p, 1, a);
            FN(orc_rforce)(seeds + 4 * (p + NN), 1, b);
            REAL *ri = r + 7 * p;
            const REAL *fi = f + 7 * p;
            ri[0] += kr * fi[0] + (REAL)P->varR * a[0];
            ri[1] += kr * fi[1] + (REAL)P->varR * a[1];
            ri[2] += kr * fi[2] + (REAL)P->varR * a[2];
            ri[3] += kfi * fi[3] + nfi * b[0];            /* fi    <- rf_ang.x */
            ri[5] += kfi * fi[5] + nfi * b[1];            /* psi   <- rf_ang.y */
            ri[4] += kth * fi[4] + (REAL)P->varTheta * b[2]; /* theta <- rf_ang.z */
        }
        for (int c = 0; c < 6; c++) f[7 * p + c] = 0;
    }
}

/* -------------------------------------------------------------------- TEA */
/* Normalised RPY block D_ij/D_ii for unit vector u and distance w
 * (integrateTea_RPY, src/bdhitea_kernel.cu:38-58): T = cii I + crr u u^T. */
static void FN(rpy)(REAL ux, REAL uy, REAL uz, REAL w, REAL a, REAL T[6]) {
    const REAL ra = w / a;
    REAL crr, cii;
    if (ra > (REAL)2) {
        crr = (REAL)0.75 / ra * ((REAL)1 - (REAL)2 / ra / ra);
        cii = (REAL)0.75 / ra * ((REAL)1 + (REAL)2 / (REAL)3 / ra / ra);
    } else {
        crr = (REAL)3 * ra / (REAL)32;
        cii = (REAL)1 - (REAL)9 * ra / (REAL)32;
    }
    T[0] = ux * ux * crr + cii; /* xx */
    T[1] = ux * uy * crr;       /* xy */
    T[2] = ux * uz * crr;       /* xz */
    T[3] = uy * uy * crr + cii; /* yy */
    T[4] = uy * uz * crr;       /* yz */
    T[5] = uz * uz * crr + cii; /* zz */
}

/* integrateTea_prepare (src/bdhitea_kernel.cu:16-36): random force of every
 * bead from stream p scaled by sqrt(2 kB T gammaR / dt); snapshots of force
 * and coordinates (4 REALs per bead); xyz of f zeroed. */
void FN(orc_tea_prepare)(const mtg_params *P, const mtg_topology *T, REAL *f, const REAL *r,
                         uint32_t *seeds, REAL *rforce, REAL *mforce, REAL *coords) {
    const size_t NN = (size_t)T->Ntot * T->Ntr;
    const REAL var = MSQRT((REAL)2 * (REAL)0.0019872041f * (REAL)P->Temp * (REAL)P->gammaR / (REAL)P->dt);
    ORC_PAR_FOR
    for (size_t p = 0; p < NN; p++) {
        REAL g[4];
        FN(orc_rforce)(seeds + 4 * p, 1, g);
        rforce[4 * p + 0] = g[0] * var;
        rforce[4 * p + 1] = g[1] * var;
        rforce[4 * p + 2] = g[2] * var;
        rforce[4 * p + 3] = g[3];
        mforce[4 * p + 0] = f[7 * p + 0];
        mforce[4 * p + 1] = f[7 * p + 1];
        mforce[4 * p + 2] = f[7 * p + 2];
        mforce[4 * p + 3] = 0;
        f[7 * p + 0] = f[7 * p + 1] = f[7 * p + 2] = 0;
        coords[4 * p + 0] = CX(r, p);
        coords[4 * p + 1] = CY(r, p);
        coords[4 * p + 2] = CZ(r, p);
        coords[4 * p + 3] = 0;
    }
}

/* integrateTea_epsilon_unlisted + _local (src/bdhitea_kernel.cu:61-101):
 * ci[4p+c] = sum_j sum_b T_cb^2 (row c), eps[p] = sum_j sum of all 9 T
 * entries, over non-extra j != p of the same trajectory (0 for extra p). */
void FN(orc_tea_epsilon)(const mtg_params *P, const mtg_topology *T, const REAL *r, REAL *ci, REAL *eps) {
    const int N = T->Ntot;
    const size_t NN = (size_t)N * T->Ntr;
    ORC_PAR_FOR
    for (size_t p = 0; p < NN; p++) {
        const size_t i0 = (p / N) * N;
        REAL sx = 0, sy = 0, sz = 0, sw = 0;
        for (size_t q = i0; q < i0 + N; q++) {
            if (q == p || T->extra[q] || T->extra[p]) continue;
            REAL dx = CX(r, q) - CX(r, p), dy = CY(r, q) - CY(r, p), dz = CZ(r, q) - CZ(r, p);
            const REAL w = MSQRT(dx * dx + dy * dy + dz * dz);
            dx /= w; dy /= w; dz /= w;
            REAL D[6];
            FN(rpy)(dx, dy, dz, w, (REAL)P->tea_a, D);
            sw += D[0] + 2 * D[1] + 2 * D[2] + D[3] + 2 * D[4] + D[5];
            sx += D[0] * D[0] + D[1] * D[1] + D[2] * D[2];
            sy += D[1] * D[1] + D[3] * D[3] + D[4] * D[4];
            sz += D[2] * D[2] + D[4] * D[4] + D[5] * D[5];
        }
        ci[4 * p + 0] = sx;
        ci[4 * p + 1] = sy;
        ci[4 * p + 2] = sz;
        ci[4 * p + 3] = 0;
        eps[p] = sw;
    }
}

/* Host reduction of updateTea (src/bdhitea.cu:57-118), FP64:
 * eps_t = sum eps_i / (3N'(3N'-3)) over the N' non-extra beads; clamp to 1
 * (error if capricious); error if > epsmax; a = (3N'-1)eps^2 - (3N'-2)eps;
 * beta = (1 - sqrt(1-a))/a, or 0.5 when |a| < 1e-7 (error if capricious and
 * tea_a > 0).  Returns 0 or MTG_E_TEA_EPS (after filling every trajectory). */
int FN(orc_tea_beta)(const mtg_params *P, const mtg_topology *T, const REAL *eps, double *eps_traj, REAL *beta) {
    const int N = T->Ntot;
    int status = 0;
    for (int t = 0; t < T->Ntr; t++) {
        int nn = 0;
        for (int j = 0; j < N; j++) nn += !T->extra[j + (size_t)N * t];
        double e = 0.0;
        for (int i = 0; i < N; i++) e += (double)eps[(size_t)t * N + i];
        e /= 3. * nn * (3. * nn - 3.);
        if (e > 1.0) {
            if (P->tea_capricious) status = MTG_E_TEA_EPS;
            e = 1.0;
        }
        if (e > P->tea_epsmax) status = MTG_E_TEA_EPS;
        const double a = (3. * nn - 1.) * e * e - (3. * nn - 2.) * e;
        if (fabs(a) < 1e-7) {
            beta[t] = (REAL)0.5f;
            if (P->tea_capricious && P->tea_a > 0.0f) status = MTG_E_TEA_EPS;
        } else {
            beta[t] = (REAL)((1. - sqrt(1. - a)) / a);
        }
        if (eps_traj) eps_traj[t] = e;
    }
    return status;
}

/* integrateTea_kernel_unlisted + integrateTea_force
 * (src/bdhitea_kernel.cu:104-213): effective force
 * F_i + C_i o R_i + sum_{j != i} D_ij/D_ii (F_j + beta C_i o R_j), xyz moved
 * by dt/gammaR times it; angles as integrate_kernel from stream p+Ntot*Ntr,
 * which is consumed for every bead. */
void FN(orc_tea_integrate)(const mtg_params *P, const mtg_topology *T, REAL *f, REAL *r, uint32_t *seeds,
                           const REAL *ci, const REAL *beta, const REAL *rforce, const REAL *mforce,
                           const REAL *coords) {
    const int N = T->Ntot;
    const size_t NN = (size_t)N * T->Ntr;
    const REAL kr = (REAL)P->dt / (REAL)P->gammaR;
    const REAL kfi = (REAL)P->dt / ((REAL)P->gammaTheta * (REAL)P->alpha);
    const REAL kth = (REAL)P->dt / (REAL)P->gammaTheta;
    const REAL nfi = (REAL)P->varTheta * MSQRT((REAL)P->freeze_temp / (REAL)P->alpha);
    ORC_PAR_FOR
    for (size_t p = 0; p < NN; p++) {
        const size_t tr = p / N, i0 = tr * N;
        const REAL b = beta[tr], b2 = b * b;
        REAL cx = (REAL)1 / MSQRT((REAL)1 + b2 * ci[4 * p + 0]);
        REAL cy = (REAL)1 / MSQRT((REAL)1 + b2 * ci[4 * p + 1]);
        REAL cz = (REAL)1 / MSQRT((REAL)1 + b2 * ci[4 * p + 2]);
        REAL fx = mforce[4 * p + 0] + rforce[4 * p + 0] * cx;
        REAL fy = mforce[4 * p + 1] + rforce[4 * p + 1] * cy;
        REAL fz = mforce[4 * p + 2] + rforce[4 * p + 2] * cz;
        cx *= b; cy *= b; cz *= b;
        const REAL xi = coords[4 * p + 0], yi = coords[4 * p + 1], zi = coords[4 * p + 2];
        for (size_t q = i0; q < i0 + N; q++) {
            if (q == p || T->extra[p] || T->extra[q]) continue;
            REAL dx = coords[4 * q + 0] - xi, dy = coords[4 * q + 1] - yi, dz = coords[4 * q + 2] - zi;
            const REAL w = MSQRT(dx * dx + dy * dy + dz * dz);
            dx /= w; dy /= w; dz /= w;
            const REAL gx = mforce[4 * q + 0] + rforce[4 * q + 0] * cx;
            const REAL gy = mforce[4 * q + 1] + rforce[4 * q + 1] * cy;
            const REAL gz = mforce[4 * q + 2] + rforce[4 * q + 2] * cz;
            REAL D[6];
            FN(rpy)(dx, dy, dz, w, (REAL)P->tea_a, D);
            fx += D[0] * gx + D[1] * gy + D[2] * gz;
            fy += D[1] * gx + D[3] * gy + D[4] * gz;
            fz += D[2] * gx + D[4] * gy + D[5] * gz;
        }
        REAL ang[4];
        FN(orc_rforce)(seeds + 4 * (p + NN), 1, ang);
        if (!T->fixed[p % N] && !T->extra[p]) {
            REAL *ri = r + 7 * p;
            const REAL *fi = f + 7 * p;
            ri[0] = xi + kr * fx;
            ri[1] = yi + kr * fy;
            ri[2] = zi + kr * fz;
            ri[3] += kfi * fi[3] + nfi * ang[0];
            ri[5] += kfi * fi[5] + nfi * ang[1];
            ri[4] += kth * fi[4] + (REAL)P->varTheta * ang[2];
        }
    }
}

/* ---------------------------------------------------------------- step loop */
/* The device part of compute()'s loop (src/compute_cuda.cu:1137-1238) for
 * steps first_step .. first_step+nsteps-1, without host I/O and updater
 * hooks.  tea_ci [4*NN] and tea_beta [Ntr] carry TEA state between calls. */
int FN(orc_run)(const mtg_params *P, const mtg_topology *T, REAL *r, REAL *f, uint32_t *seeds, int maxLong,
                int *longCount, int *lon, int maxLat, int *latCount, int *lat, int maxLJ, int *LJCount,
                int *LJ, long long first_step, int nsteps, REAL *tea_ci, REAL *tea_beta) {
    const size_t NN = (size_t)T->Ntot * T->Ntr;
    int status = 0, overflow = 0;
    REAL *rf = NULL, *mf = NULL, *cs = NULL, *eps = NULL;
    if (P->hdi_on) {
        rf = (REAL *)malloc(sizeof(REAL) * 4 * NN);
        mf = (REAL *)malloc(sizeof(REAL) * 4 * NN);
        cs = (REAL *)malloc(sizeof(REAL) * 4 * NN);
        eps = (REAL *)malloc(sizeof(REAL) * NN);
    }
    for (long long step = first_step; step < first_step + nsteps; step++) {
        if (step % P->ljpairsupdatefreq == 0) {
            if (P->lj_on) FN(orc_lj_list)(P, T, r, maxLJ, LJCount, LJ, &overflow);
            if (P->is_assembly) FN(orc_pairs_list)(P, T, r, maxLong, longCount, lon, maxLat, latCount, lat, &overflow);
        }
        FN(orc_forces)(P, T, r, maxLong, longCount, lon, maxLat, latCount, lat, maxLJ, LJCount, LJ, f);
        if (P->hdi_on) {
            if (step % P->tea_epsilon_freq == 0) {
                FN(orc_tea_epsilon)(P, T, r, tea_ci, eps);
                const int s = FN(orc_tea_beta)(P, T, eps, NULL, tea_beta);
                if (s && !status) status = s;
            }
            FN(orc_tea_prepare)(P, T, f, r, seeds, rf, mf, cs);
            FN(orc_tea_integrate)(P, T, f, r, seeds, tea_ci, tea_beta, rf, mf, cs);
        } else {
            FN(orc_integrate)(P, T, r, f, seeds);
        }
    }
    free(rf);
    free(mf);
    free(cs);
    free(eps);
    if (overflow && !status) status = MTG_E_OVERFLOW;
    return status;
}

#undef V3
#undef FRAME
#undef ACC
#undef FN
#undef CAT
#undef CAT2
