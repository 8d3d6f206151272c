// energy_noalloc.cu - per-trajectory energy totals without any allocation.
//
// mtg_energies() reduces the per-bead energies through block partial sums
// kept in a buffer the engine allocated.  This file offers the same
// reduction for callers that must not allocate device memory at the moment
// they ask for energies: analysis hooks that run while other engines on the
// same GPU have work in flight (cudaMalloc and cudaFree may synchronise the
// whole device and stall that work), and processes whose device memory is
// reserved up front by a pool allocator, where a fresh cudaMalloc can fail.
// Its scratch (the block partials) lives in a fixed, file-scope device array
// instead, so the call itself allocates nothing.
#include "mtg_engine.cuh"

namespace {

// Block partials: 7 doubles per 128-bead chunk; 16384 chunks = up to
// 2,097,152 beads per call, 917,504 bytes held on every GPU that loads the
// library, until the process exits.
constexpr int kMaxChunks = 16384;
static __device__ __align__(256) double g_energy_scratch[kMaxChunks * MTG_ENERGY_TERMS];

// Device address of g_energy_scratch in the current context.  The host-side
// symbol is only a stand-in; a kernel needs this address.  It is looked up
// once per engine (the engine's first call, with its device current) and kept
// in the engine: an engine's buffers and this address belong to the same
// context, so an engine created after the context was torn down and rebuilt
// (cudaDeviceReset) looks the address up again instead of reusing a stale one.
int scratch_address(mtg_engine *e, double **out) {
    if (!e->noalloc_scratch) {
        void *p = nullptr;
        const cudaError_t err = cudaGetSymbolAddress(&p, g_energy_scratch);
        if (err != cudaSuccess)
            return mtg_internal_fail(MTG_E_CUDA, "mtg_energies_noalloc: cudaGetSymbolAddress of the scratch failed");
        e->noalloc_scratch = static_cast<double *>(p);
    }
    *out = e->noalloc_scratch;
    return MTG_OK;
}

// Puts the caller's current device back on every return path.
struct DeviceGuard {
    int prev = -1;
    DeviceGuard() {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    }
    ~DeviceGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

}  // namespace

extern "C" int mtg_energies_noalloc(mtg_engine *e, double *d_per_traj) {
    if (!e || !d_per_traj) return mtg_internal_fail(MTG_E_CONFIG, "mtg_energies_noalloc: engine or output is NULL");
    if (!e->have_state) return mtg_internal_fail(MTG_E_STATE, "mtg_energies_noalloc: no state uploaded");
    if (e->nwork > kMaxChunks)
        return mtg_internal_fail(MTG_E_CONFIG,
                                 "mtg_energies_noalloc: the batch needs more than 16384 chunks of 128 beads "
                                 "(trajectories are chunked separately); use mtg_energies");
    DeviceGuard guard;
    // an error left by earlier work of this thread is reported as such and
    // left in place (peek, not get), so it is neither cleared nor blamed on
    // this call's launches
    const cudaError_t pending = cudaPeekAtLastError();
    if (pending != cudaSuccess)
        return mtg_internal_fail(MTG_E_CUDA, "mtg_energies_noalloc: a CUDA error was pending before the call "
                                             "(left unreported by this call's launches)");
    if (cudaSetDevice(e->device) != cudaSuccess)
        return mtg_internal_fail(MTG_E_CUDA, "mtg_energies_noalloc: cudaSetDevice failed");
    double *scratch = nullptr;
    const int rc = scratch_address(e, &scratch);
    if (rc != MTG_OK) return rc;
    // every chunk's partials are overwritten by the energy kernel before the
    // totals kernel reads them, so nothing needs clearing between calls
    mtg::launch_energy(e->kp, e->bufs(), nullptr, scratch, e->work, e->nwork, e->stream);
    if (cudaGetLastError() != cudaSuccess)
        return mtg_internal_fail(MTG_E_CUDA, "mtg_energies_noalloc: energy kernel launch failed");
    mtg::launch_energy_totals(e->kp, scratch, e->work_first, d_per_traj, e->err, e->stream);
    if (cudaGetLastError() != cudaSuccess)
        return mtg_internal_fail(MTG_E_CUDA, "mtg_energies_noalloc: totals kernel launch failed");
    return MTG_OK;
}
