/*
 * mt_oracle.c - CPU oracle for the MADDY Brownian/Langevin hot path.
 *
 * TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
 * CPU-baseline legs of bench.py, as the reference to compare against, never
 * as the product path.  Built with
 * -ffp-contract=off so that the FP32 results are identical on x86-64 and
 * aarch64 hosts.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <limits.h>
#include "mt_oracle.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* Each bead's outputs depend only on its own inputs, so the per-bead loops
 * run in parallel (OpenMP) with results independent of the thread count. */
#ifdef _OPENMP
#define ORC_PAR_FOR _Pragma("omp parallel for schedule(dynamic, 16)")
#define ORC_SET_FLAG(x) do { _Pragma("omp atomic write") (x) = 1; } while (0)
#else
#define ORC_PAR_FOR
#define ORC_SET_FLAG(x) ((x) = 1)
#endif

/* ------------------------------------------------------------------ ran2 */
/* Numerical Recipes ran2 (L'Ecuyer with Bays-Durham shuffle) as used by the
 * reference seeding, src/ran2.h:18-56.  The reference keeps idum2, iy and
 * iv[] in function statics; a fresh process starts them at 123456789, 0 and
 * zeros, which is what each orc_generate_seeds() call reproduces. */
typedef struct {
    int idum2, iy, iv[32];
} ran2_state;

static double ran2(int *idum, ran2_state *st) {
    const int IM1 = 2147483563, IM2 = 2147483399, IMM1 = IM1 - 1;
    const int IA1 = 40014, IA2 = 40692, IQ1 = 53668, IQ2 = 52774, IR1 = 12211, IR2 = 3791;
    const int NTAB = 32, NDIV = 1 + IMM1 / NTAB;
    const double AM = 1.0 / IM1, RNMX = 1.0 - 1.2e-7;
    int j, k;
    if (*idum <= 0) {
        *idum = (-(*idum) < 1) ? 1 : -(*idum);
        st->idum2 = *idum;
        for (j = NTAB + 7; j >= 0; j--) {
            k = *idum / IQ1;
            *idum = IA1 * (*idum - k * IQ1) - k * IR1;
            if (*idum < 0) *idum += IM1;
            if (j < NTAB) st->iv[j] = *idum;
        }
        st->iy = st->iv[0];
    }
    k = *idum / IQ1;
    *idum = IA1 * (*idum - k * IQ1) - k * IR1;
    if (*idum < 0) *idum += IM1;
    k = st->idum2 / IQ2;
    st->idum2 = IA2 * (st->idum2 - k * IQ2) - k * IR2;
    if (st->idum2 < 0) st->idum2 += IM2;
    j = st->iy / NDIV;
    st->iy = st->iv[j] - st->idum2;
    st->iv[j] = *idum;
    if (st->iy < 1) st->iy += IMM1;
    const double t = AM * st->iy;
    return t > RNMX ? RNMX : t;
}

/* generateSeeds (src/HybridTaus.cu:32-48): each uint4 component drawn as
 * (unsigned)(ran2 * UINT_MAX), redrawn while < 128. */
void orc_generate_seeds(int seed, int Np, uint32_t *seeds) {
    ran2_state st;
    st.idum2 = 123456789;
    st.iy = 0;
    memset(st.iv, 0, sizeof(st.iv));
    for (int i = 0; i < Np; i++) {
        for (int c = 0; c < 4; c++) {
            uint32_t v;
            do {
                v = (uint32_t)(ran2(&seed, &st) * (double)UINT_MAX);
            } while (v < 128u);
            seeds[4 * i + c] = v;
        }
    }
}

/* HybridTaus (src/HybridTaus.cu:63-82, GPU Gems 3 ch. 37): three Tausworthe
 * steps and one LCG step, XOR-combined. */
static uint32_t taus_step(uint32_t *z, int S1, int S2, int S3, uint32_t M) {
    const uint32_t b = ((*z << S1) ^ *z) >> S2;
    return *z = ((*z & M) << S3) ^ b;
}

uint32_t orc_hybrid_taus(uint32_t *s) {
    const uint32_t a = taus_step(&s[0], 13, 19, 12, 4294967294u);
    const uint32_t b = taus_step(&s[1], 2, 25, 4, 4294967288u);
    const uint32_t c = taus_step(&s[2], 3, 11, 17, 4294967280u);
    s[3] = 1664525u * s[3] + 1013904223u;
    return a ^ b ^ c ^ s[3];
}

/* uintToFloat (src/HybridTaus.cu:53-61): mantissa bits into [1,2) minus 1,
 * an exact 0 mapped to 1e-8. */
float orc_uint_to_float(uint32_t u) {
    const uint32_t bits = 0x3f800000u | (0x007fffffu & u);
    float f;
    memcpy(&f, &bits, sizeof f);
    f -= 1.0f;
    return f == 0.0f ? 1.0e-8f : f;
}

/* ---------------------------------------------------------- FP32 oracle */
#define REAL float
#define SUF f32
#define MSQRT sqrtf
#define MSIN sinf
#define MCOS cosf
#define MEXP expf
#define MLOG logf
#define MFABS fabsf
#include "mt_oracle_impl.h"
#undef REAL
#undef SUF
#undef MSQRT
#undef MSIN
#undef MCOS
#undef MEXP
#undef MLOG
#undef MFABS

/* ---------------------------------------------------------- FP64 oracle */
#define REAL double
#define SUF f64
#define MSQRT sqrt
#define MSIN sin
#define MCOS cos
#define MEXP exp
#define MLOG log
#define MFABS fabs
#include "mt_oracle_impl.h"
