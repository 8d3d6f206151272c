// restart.cu - bit-exact restart of an engine: one binary file with the
// complete dynamic state, so that a run resumed from it reproduces the
// uninterrupted run bit for bit.
//
// The reference's writeRestart/readRestart (src/preparator.cpp:664-714) keep
// x, y, z, fi, psi, theta as "%f" text (XYZ files) and re-seed the noise, so a
// resumed reference run follows another trajectory.  This file adds what that
// restart lacks: the bead state in full precision, the HybridTaus states of
// both streams of every bead, the per-bead flag words (gtp / extra /
// on_tubule as changed since creation), the neighbour lists of the current
// pair-list period, and the TEA state (C_i row sums, beta, epsilon of the
// last epsilon step).
//
// Layout (little-endian):
//   "MTGRST\0\1"  int32 version(1)  int32 nb, nt, hdi_on, maxLJ, maxLong,
//   maxLat, lists_valid   int64 step
//   f32 coords[7 nb]   i32 flags[nb]   u32 seeds[8 nb]
//   if lists_valid: i32 ljc[nb], lj[maxLJ nb], lonc[nb], lon[maxLong nb],
//                   latc[nb], lat[maxLat nb]   (k-major, as on the device)
//   if hdi_on:      f32 tea_ci[4 nb], tea_beta[nt]   f64 tea_eps_t[nt]
//   u64 FNV-1a hash of every byte before it
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "mtg_engine.cuh"

namespace {

constexpr char kMagic[8] = {'M', 'T', 'G', 'R', 'S', 'T', 0, 1};
constexpr int32_t kVersion = 1;

struct Fnv {
    uint64_t h = 1469598103934665603ull;
    void add(const void *p, size_t n) {
        const unsigned char *c = static_cast<const unsigned char *>(p);
        for (size_t i = 0; i < n; i++) h = (h ^ c[i]) * 1099511628211ull;
    }
};

struct Writer {
    FILE *f;
    Fnv fnv;
    bool ok = true;
    void put(const void *p, size_t n) {
        if (!ok || n == 0) return;
        ok = std::fwrite(p, 1, n, f) == n;
        fnv.add(p, n);
    }
};

struct Reader {
    FILE *f;
    Fnv fnv;
    bool ok = true;
    void get(void *p, size_t n) {
        if (!ok || n == 0) return;
        ok = std::fread(p, 1, n, f) == n;
        if (ok) fnv.add(p, n);
    }
};

struct Header {
    int32_t version, nb, nt, hdi, max_lj, max_long, max_lat, lists_valid;
    int64_t step;
};

int cuda_fail(cudaError_t e) { return mtg_internal_fail(MTG_E_CUDA, cudaGetErrorString(e)); }

// device -> host bytes
template <typename T>
int d2h(std::vector<T> &h, const void *d, size_t n, cudaStream_t s) {
    h.resize(n);
    const cudaError_t e = cudaMemcpyAsync(h.data(), d, sizeof(T) * n, cudaMemcpyDeviceToHost, s);
    return e == cudaSuccess ? MTG_OK : cuda_fail(e);
}
template <typename T>
int h2d(void *d, const std::vector<T> &h, cudaStream_t s) {
    const cudaError_t e = cudaMemcpyAsync(d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, s);
    return e == cudaSuccess ? MTG_OK : cuda_fail(e);
}

}  // namespace

extern "C" {

int mtg_write_restart(mtg_engine *e, const char *path, long long step) {
    if (!e || !path) return mtg_internal_fail(MTG_E_CONFIG, "engine or path is NULL");
    if (!e->have_state) return mtg_internal_fail(MTG_E_STATE, "no state uploaded");
    cudaSetDevice(e->device);
    const size_t nb = e->nb, nt = e->nt;
    std::vector<float> coords(7 * nb);
    int rc = mtg_download_state(e, coords.data(), nullptr);
    if (rc) return rc;
    std::vector<int32_t> flags, ljc, lj, lonc, lon, latc, lat;
    std::vector<uint32_t> seeds;
    std::vector<float> ci, beta;
    std::vector<double> eps_t;
    const Header H{kVersion, e->nb, e->nt, e->p.hdi_on ? 1 : 0, e->kp.maxLJ, e->kp.maxLong, e->kp.maxLat,
                   e->lists_valid ? 1 : 0, (int64_t)step};
    if ((rc = d2h(flags, e->flags, nb, e->stream)) || (rc = d2h(seeds, e->seeds, 8 * nb, e->stream))) return rc;
    if (H.lists_valid &&
        ((rc = d2h(ljc, e->ljc, nb, e->stream)) || (rc = d2h(lj, e->lj, (size_t)H.max_lj * nb, e->stream)) ||
         (rc = d2h(lonc, e->lonc, nb, e->stream)) || (rc = d2h(lon, e->lon, (size_t)H.max_long * nb, e->stream)) ||
         (rc = d2h(latc, e->latc, nb, e->stream)) || (rc = d2h(lat, e->lat, (size_t)H.max_lat * nb, e->stream))))
        return rc;
    if (H.hdi && ((rc = d2h(ci, e->tea_ci, 4 * nb, e->stream)) || (rc = d2h(beta, e->tea_beta, nt, e->stream)) ||
                  (rc = d2h(eps_t, e->tea_eps_t, nt, e->stream))))
        return rc;
    const cudaError_t ce = cudaStreamSynchronize(e->stream);
    if (ce != cudaSuccess) return cuda_fail(ce);

    FILE *f = std::fopen(path, "wb");
    if (!f) return mtg_internal_fail(MTG_E_CONFIG, "cannot open the restart file for writing");
    Writer w{f};
    w.put(kMagic, sizeof kMagic);
    w.put(&H, sizeof H);
    w.put(coords.data(), sizeof(float) * coords.size());
    w.put(flags.data(), sizeof(int32_t) * flags.size());
    w.put(seeds.data(), sizeof(uint32_t) * seeds.size());
    if (H.lists_valid) {
        for (auto *v : {&ljc, &lj, &lonc, &lon, &latc, &lat}) w.put(v->data(), sizeof(int32_t) * v->size());
    }
    if (H.hdi) {
        w.put(ci.data(), sizeof(float) * ci.size());
        w.put(beta.data(), sizeof(float) * beta.size());
        w.put(eps_t.data(), sizeof(double) * eps_t.size());
    }
    const uint64_t hash = w.fnv.h;
    if (w.ok) w.ok = std::fwrite(&hash, sizeof hash, 1, f) == 1;
    const bool closed = std::fclose(f) == 0;
    if (!w.ok || !closed) return mtg_internal_fail(MTG_E_CONFIG, "writing the restart file failed");
    return MTG_OK;
}

int mtg_read_restart(mtg_engine *e, const char *path, long long *step) {
    if (!e || !path) return mtg_internal_fail(MTG_E_CONFIG, "engine or path is NULL");
    cudaSetDevice(e->device);
    FILE *f = std::fopen(path, "rb");
    if (!f) return mtg_internal_fail(MTG_E_CONFIG, "cannot open the restart file");
    Reader r{f};
    char magic[8];
    Header H{};
    r.get(magic, sizeof magic);
    r.get(&H, sizeof H);
    const size_t nb = e->nb, nt = e->nt;
    if (!r.ok || std::memcmp(magic, kMagic, sizeof magic) != 0 || H.version != kVersion) {
        std::fclose(f);
        return mtg_internal_fail(MTG_E_CONFIG, "not a restart file of this format");
    }
    if (H.nb != e->nb || H.nt != e->nt || H.hdi != (e->p.hdi_on ? 1 : 0) || H.max_lj != e->kp.maxLJ ||
        H.max_long != e->kp.maxLong || H.max_lat != e->kp.maxLat) {
        std::fclose(f);
        return mtg_internal_fail(MTG_E_CONFIG, "the restart file belongs to another system (sizes or modes differ)");
    }
    std::vector<float> coords(7 * nb), ci, beta;
    std::vector<int32_t> flags(nb), ljc, lj, lonc, lon, latc, lat;
    std::vector<uint32_t> seeds(8 * nb);
    std::vector<double> eps_t;
    r.get(coords.data(), sizeof(float) * coords.size());
    r.get(flags.data(), sizeof(int32_t) * flags.size());
    r.get(seeds.data(), sizeof(uint32_t) * seeds.size());
    if (H.lists_valid) {
        ljc.resize(nb);
        lj.resize((size_t)H.max_lj * nb);
        lonc.resize(nb);
        lon.resize((size_t)H.max_long * nb);
        latc.resize(nb);
        lat.resize((size_t)H.max_lat * nb);
        for (auto *v : {&ljc, &lj, &lonc, &lon, &latc, &lat}) r.get(v->data(), sizeof(int32_t) * v->size());
    }
    if (H.hdi) {
        ci.resize(4 * nb);
        beta.resize(nt);
        eps_t.resize(nt);
        r.get(ci.data(), sizeof(float) * ci.size());
        r.get(beta.data(), sizeof(float) * beta.size());
        r.get(eps_t.data(), sizeof(double) * eps_t.size());
    }
    const uint64_t hash = r.fnv.h;
    uint64_t stored = 0;
    const bool tail = r.ok && std::fread(&stored, sizeof stored, 1, f) == 1;
    std::fclose(f);
    if (!tail || stored != hash) return mtg_internal_fail(MTG_E_CONFIG, "the restart file is truncated or corrupt");

    int rc = mtg_upload_state(e, coords.data());
    if (rc) return rc;
    if ((rc = h2d(e->flags, flags, e->stream)) || (rc = h2d(e->seeds, seeds, e->stream))) return rc;
    if (H.lists_valid && ((rc = h2d(e->ljc, ljc, e->stream)) || (rc = h2d(e->lj, lj, e->stream)) ||
                          (rc = h2d(e->lonc, lonc, e->stream)) || (rc = h2d(e->lon, lon, e->stream)) ||
                          (rc = h2d(e->latc, latc, e->stream)) || (rc = h2d(e->lat, lat, e->stream))))
        return rc;
    if (H.hdi && ((rc = h2d(e->tea_ci, ci, e->stream)) || (rc = h2d(e->tea_beta, beta, e->stream)) ||
                  (rc = h2d(e->tea_eps_t, eps_t, e->stream))))
        return rc;
    const cudaError_t ce = cudaStreamSynchronize(e->stream);
    if (ce != cudaSuccess) return cuda_fail(ce);
    e->lists_valid = H.lists_valid != 0;
    e->lists_fresh = false;
    if (step) *step = H.step;
    return MTG_OK;
}

}  // extern "C"
