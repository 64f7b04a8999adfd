// lbm_staged.cu -- the fused collide-stream step with tensor-memory-access
// (TMA) staging of the pulled rows, warp-specialised.
//
// A tile is TX x TY cells of one z plane (TX * TY = 256 consumer threads,
// one cell each).  For every population l, one tiled cp.async.bulk.tensor
// copy brings the tile's source box -- TY rows shifted by (-c_y, -c_z),
// widened by one 16-byte group on the side a c_x link comes from -- into
// shared memory, so a thread reads its 19 (+7) pulled values at offsets
// fixed at compile time.  Boxes reaching outside the lattice are zero-filled
// by the copy engine; the lanes on a domain face redo exactly their
// face-crossing links with the boundary-class rules from global memory.  The
// updated populations go to a shared output tile and leave with one tensor
// store per population.
//
// A ninth warp produces: it issues the boxes of tile k+3 as soon as the
// consumers have released the input stage of tile k, stores tile k's output
// stage, and hands that stage back once the store has read it.  Consumers
// and producer meet only on mbarriers (full / consumed / output-free), so no
// block-wide barrier sits in the loop.  Every wait is bounded; a thread whose
// wait gives up sets ST_TIMEOUT and leaves.
//
// With region = 1 the tiles of the near box are skipped (k_step covers
// them).
#include <cuda.h>

#include <algorithm>

#include "lbm_internal.h"
#include "lbm_step.cuh"

namespace lbmk {

constexpr int kStThreads = 256;                  // consumers: one cell of the tile each
constexpr int kStBlock = kStThreads + 32;        // + the producer warp
constexpr int kStIn = 3;                          // input stages
constexpr int kStOut = 2;                         // output stages (tensor-store mode)
// Output written by the consumers with plain stores (faster as measured);
// true routes it through kStOut shared output stages and tensor stores.
constexpr bool kStTmaStore = false;
constexpr long long kStWaitLimit = 1ll << 22;     // tests of a bounded mbarrier wait

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Bounded wait for the phase of `bar` with this parity.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    for (long long it = 0; it < kStWaitLimit; it++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// 4-D tiled tensor copies: coordinates (x, y, z, population).
__device__ __forceinline__ void tma_load4(void *dst, const CUtensorMap *map, int x, int y, int z, int l,
                                          uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
        "%5}], [%6];" ::"r"(smem_u32(dst)),
        "l"(map), "r"(x), "r"(y), "r"(z), "r"(l), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tma_store4(const CUtensorMap *map, int x, int y, int z, int l, const void *src) {
    asm volatile("cp.async.bulk.tensor.4d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3, %4}], [%5];" ::"l"(map),
                 "r"(x), "r"(y), "r"(z), "r"(l), "r"(smem_u32(src))
                 : "memory");
}

__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read_all() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void bulk_wait_read_keep() {
    asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(N) : "memory");
}
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// One lane of the (fully active) warp.
__device__ __forceinline__ bool elect_one() {
    uint32_t e = 0;
    asm volatile(
        "{\n\t.reg .pred p;\n\telect.sync _|p, 0xffffffff;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(e));
    return e != 0;
}

// Shared-memory geometry of one tile, all compile-time.
template <class T, int TX, bool THERMAL>
struct StGeom {
    static constexpr int TY = kStThreads / TX;
    static constexpr int H = 16 / (int)sizeof(T);  // elements in one 16-byte group
    static constexpr int NQ = THERMAL ? Q + QT : Q;
    // population q of a stage: link l = q (flow) or q - Q (heat)
    static constexpr __host__ __device__ int link(int q) { return q < Q ? q : q - Q; }
    static constexpr __host__ __device__ int width(int q) { return TX + (cx(link(q)) != 0 ? H : 0); }
    static constexpr __host__ __device__ int box_bytes(int q) { return width(q) * TY * (int)sizeof(T); }
    static constexpr __host__ __device__ int padded(int b) { return (b + 127) / 128 * 128; }
    static constexpr __host__ __device__ int in_off(int q) {
        int o = 0;
        for (int p = 0; p < q; p++) o += padded(box_bytes(p));
        return o;
    }
    static constexpr __host__ __device__ uint32_t tx_bytes() {
        uint32_t b = 0;
        for (int p = 0; p < NQ; p++) b += (uint32_t)box_bytes(p);
        return b;
    }
    static constexpr int IN_BYTES = in_off(NQ);                       // one input stage
    static constexpr int OUT_BYTES = NQ * TX * TY * (int)sizeof(T);  // one output stage
    // input stages, output stages, mbarriers, tile records
    static constexpr size_t SMEM = 128 + kStIn * (size_t)IN_BYTES + (kStTmaStore ? kStOut * (size_t)OUT_BYTES : 0) +
                                   (2 * kStIn + kStOut) * 8 + kStIn * 16;
};

enum { TILE_STAGED = 0, TILE_SKIP = 1 };

template <int TX, int TY>
__device__ __forceinline__ int4 tile_of(long long t, long long ntiles, int tiles_x, int tiles_y, const StepParams &P,
                                        int region) {
    if (t >= ntiles) return make_int4(0, 0, 0, TILE_SKIP);
    const long long row = t / tiles_x;
    const int x0 = (int)(t - row * tiles_x) * TX;
    const int z = (int)(row / tiles_y);
    const int y0 = (int)(row - (long long)z * tiles_y) * TY;
    int kind = TILE_STAGED;
    if (region == 1 && x0 >= P.nlo[0] && x0 < P.nhi[0] && y0 >= P.nlo[1] && y0 < P.nhi[1] && z >= P.nlo[2] &&
        z < P.nhi[2])
        kind = TILE_SKIP;
    return make_int4(x0, y0, z, kind);
}

template <class T, int TX, bool THERMAL, bool FORCED>
__global__ void __launch_bounds__(kStBlock) k_step_st(
    const __grid_constant__ CUtensorMap mAn, const __grid_constant__ CUtensorMap mAw,
    const __grid_constant__ CUtensorMap mB, const __grid_constant__ CUtensorMap mGn,
    const __grid_constant__ CUtensorMap mGw, const __grid_constant__ CUtensorMap mGB, const T *__restrict__ A,
    const T *__restrict__ GA, T *__restrict__ B, T *__restrict__ GB, const __grid_constant__ StepParams P,
    DevState *__restrict__ ds,
    float *__restrict__ band, int region, int tiles_x, int tiles_y, long long ntiles) {
    typedef StGeom<T, TX, THERMAL> G;
    constexpr int TY = G::TY, H = G::H, NQ = G::NQ;
    extern __shared__ unsigned char smem_raw[];
    unsigned char *smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
    unsigned char *sin = smem;                          // [kStIn][IN_BYTES]
    unsigned char *sout = smem + kStIn * G::IN_BYTES;  // [kStOut][OUT_BYTES]
    uint64_t *full = reinterpret_cast<uint64_t *>(sout + (kStTmaStore ? kStOut * G::OUT_BYTES : 0));  // boxes landed
    uint64_t *consumed = full + kStIn;    // [kStIn] consumers done with the tile
    uint64_t *ofree = consumed + kStIn;   // [kStOut] output stage read by its store
    int4 *meta = reinterpret_cast<int4 *>(ofree + kStOut);  // [kStIn] tile records

    const int tid = threadIdx.x;
    const long long G0 = blockIdx.x, GS = gridDim.x;
    const long long nk = G0 < ntiles ? (ntiles - G0 + GS - 1) / GS : 0;

    if (tid == 0) {
        for (int i = 0; i < kStIn; i++) {
            mbar_init(&full[i], 1);
            mbar_init(&consumed[i], kStThreads / 32);
        }
        for (int i = 0; i < kStOut; i++) mbar_init(&ofree[i], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    if (tid >= kStThreads) {
        // ------------------------------ producer ------------------------------
        // The whole warp runs the loop on warp-uniform values (tile index,
        // coordinates); one elected lane issues the copies.
        const bool leader = elect_one();
        // record tile k in its slot, arm full[] with its bytes, issue its boxes
        auto issue = [&](long long k) {
            const int b = (int)(k % kStIn);
            const int4 m = tile_of<TX, TY>(G0 + k * GS, ntiles, tiles_x, tiles_y, P, region);
            if (!leader) return;
            meta[b] = m;
            if (m.w != TILE_STAGED) {
                mbar_arrive_expect_tx(&full[b], 0u);
                return;
            }
            fence_proxy_async();
            mbar_arrive_expect_tx(&full[b], G::tx_bytes());
            unsigned char *stage = sin + b * G::IN_BYTES;
#pragma unroll
            for (int q = 0; q < NQ; q++) {
                const int l = G::link(q);
                const CUtensorMap *map = q < Q ? (cx(l) != 0 ? &mAw : &mAn) : (cx(l) != 0 ? &mGw : &mGn);
                tma_load4(stage + G::in_off(q), map, m.x - (cx(l) > 0 ? H : 0), m.y - cy(l), m.z - cz(l), l,
                          &full[b]);
            }
        };
        for (long long k = 0; k < kStIn && k < nk; k++) issue(k);
        for (long long k = 0; k < nk; k++) {
            const int b = (int)(k % kStIn);
            if (!__all_sync(0xffffffffu, mbar_wait(&consumed[b], (uint32_t)((k / kStIn) & 1)))) {
                if (leader) atomicOr(&ds->status, ST_TIMEOUT);
                break;
            }
            const int4 m = tile_of<TX, TY>(G0 + k * GS, ntiles, tiles_x, tiles_y, P, region);
            if (kStTmaStore && leader) {
                if (m.w == TILE_STAGED) {
                    fence_proxy_async();
                    const unsigned char *out = sout + (k % kStOut) * G::OUT_BYTES;
#pragma unroll
                    for (int q = 0; q < NQ; q++)
                        tma_store4(q < Q ? &mB : &mGB, m.x, m.y, m.z, G::link(q),
                                   out + q * TX * TY * (int)sizeof(T));
                }
                bulk_commit();
            }
            if (k + kStIn < nk) issue(k + kStIn);
            // hand back the output stage of tile k - kStOut + 1 once its store
            // has read it (the stores of the newer tiles stay in flight)
            if (kStTmaStore && k >= kStOut - 1 && leader) {
                bulk_wait_read_keep<kStOut - 1>();
                mbar_arrive(&ofree[(k - kStOut + 1) % kStOut]);
            }
        }
        if (kStTmaStore && leader) bulk_wait_all();
        return;
    }

    // ------------------------------- consumers --------------------------------
    const int tx = tid % TX, ty = tid / TX;
    const int pm = periodic_mask(P);
    for (long long k = 0; k < nk; k++) {
        const int b = (int)(k % kStIn);
        bool ok = mbar_wait(&full[b], (uint32_t)((k / kStIn) & 1));
        if (kStTmaStore && ok && k >= kStOut)
            ok = mbar_wait(&ofree[k % kStOut], (uint32_t)(((k / kStOut) - 1) & 1));
        // a warp leaves together: the per-warp arrivals below stay whole
        if (!__all_sync(0xffffffffu, ok)) {
            if ((tid & 31) == 0) atomicOr(&ds->status, ST_TIMEOUT);
            return;
        }
        const int4 m = meta[b];
        if (m.w == TILE_STAGED) {
            const int x = m.x + tx, y = m.y + ty, z = m.z;
            const long long cell = (long long)x + (long long)P.nx * ((long long)y + (long long)P.ny * z);
            const unsigned char *stage = sin + b * G::IN_BYTES;
            float f[Q], g[QT];
#pragma unroll
            for (int l = 0; l < Q; l++) {
                const T *row = reinterpret_cast<const T *>(stage + G::in_off(l)) + ty * G::width(l);
                f[l] = St<T>::lds(row + tx - cx(l) + (cx(l) > 0 ? H : 0));
            }
            if (THERMAL) {
#pragma unroll
                for (int l = 0; l < QT; l++) {
                    const T *row = reinterpret_cast<const T *>(stage + G::in_off(Q + l)) + ty * G::width(Q + l);
                    g[l] = St<T>::lds(row + tx - cx(l) + (cx(l) > 0 ? H : 0));
                }
            }
            // lanes on a domain face: the links crossing it follow the
            // boundary-class rules (the staged value there is a fill)
            const int raw = (x == 0 ? 1 : 0) | (x == P.nx - 1 ? 2 : 0) | (y == 0 ? 4 : 0) | (y == P.ny - 1 ? 8 : 0) |
                            (z == 0 ? 16 : 0) | (z == P.nz - 1 ? 32 : 0);
            if (raw) {
                const ClassEntry &ce = P.cls[raw & ~pm];
#pragma unroll
                for (int l = 1; l < Q; l++) {
                    const int cross = (cx(l) > 0 ? 1 : 0) | (cx(l) < 0 ? 2 : 0) | (cy(l) > 0 ? 4 : 0) |
                                      (cy(l) < 0 ? 8 : 0) | (cz(l) > 0 ? 16 : 0) | (cz(l) < 0 ? 32 : 0);
                    if (raw & cross) f[l] = pull_link<T>(A, l, x, y, z, cell, ce, P);
                }
                if (THERMAL) {
#pragma unroll
                    for (int l = 1; l < QT; l++) {
                        const int cross = (cx(l) > 0 ? 1 : 0) | (cx(l) < 0 ? 2 : 0) | (cy(l) > 0 ? 4 : 0) |
                                          (cy(l) < 0 ? 8 : 0) | (cz(l) > 0 ? 16 : 0) | (cz(l) < 0 ? 32 : 0);
                        if (raw & cross) g[l] = pull_heat_link<T>(GA, l, x, y, z, cell, ce, P);
                    }
                }
            }
            update_cell<T, THERMAL, FORCED>(f, g, x, y, z, cell, true, 1, 0, P, ds, nullptr, band, region != 1);
            if (kStTmaStore) {
                T *so = reinterpret_cast<T *>(sout + (k % kStOut) * G::OUT_BYTES) + ty * TX + tx;
#pragma unroll
                for (int l = 0; l < Q; l++) St<T>::st(so + l * TY * TX, f[l]);
                if (THERMAL) {
#pragma unroll
                    for (int l = 0; l < QT; l++) St<T>::st(so + (Q + l) * TY * TX, g[l]);
                }
                // this thread's output writes, visible to the tensor store
                fence_proxy_async();
            } else {
                const unsigned c = (unsigned)cell;
#pragma unroll
                for (int l = 0; l < Q; l++) St<T>::st(B + (c + P.sofs32[l]), f[l]);
                if (THERMAL) {
#pragma unroll
                    for (int l = 0; l < QT; l++) St<T>::st(GB + (c + P.sofs32[l]), g[l]);
                }
            }
        }
        __syncwarp();
        if ((tid & 31) == 0) mbar_arrive(&consumed[b]);
    }
}

// ---------------------------------------------------------------------------
// Host side: tensor maps and launch plan.
// ---------------------------------------------------------------------------
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
        cudaGetLastError();
    }
    return fn;
}

// Map of npop population arrays of stride S as a 4-D tensor (x, y, z,
// population) read or written in boxes of (box_x, box_y, 1, 1).
static bool make_map(CUtensorMap *map, int storage, void *base, const StepParams &P, int npop, int box_x,
                     int box_y) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return false;
    const size_t es = storage == 0 ? 4 : 2;
    const CUtensorMapDataType dt = storage == 0   ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32
                                   : storage == 1 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16
                                                  : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
    cuuint64_t dims[4] = {(cuuint64_t)P.nx, (cuuint64_t)P.ny, (cuuint64_t)P.nz, (cuuint64_t)npop};
    cuuint64_t strides[3] = {(cuuint64_t)P.nx * es, (cuuint64_t)P.nx * P.ny * es, (cuuint64_t)P.S * es};
    cuuint32_t box[4] = {(cuuint32_t)box_x, (cuuint32_t)box_y, 1, 1};
    cuuint32_t estr[4] = {1, 1, 1, 1};
    return fn(map, dt, 4, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <class T, int TX, bool THERMAL, bool FORCED>
static cudaError_t plan_one(int &per_sm) {
    const size_t smem = StGeom<T, TX, THERMAL>::SMEM;
    cudaError_t e =
        cudaFuncSetAttribute(k_step_st<T, TX, THERMAL, FORCED>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_step_st<T, TX, THERMAL, FORCED>, kStBlock, smem);
}

template <class T, int TX>
static cudaError_t plan_tx(bool thermal, bool forced, int &per_sm, size_t &smem) {
    if (thermal) {
        smem = StGeom<T, TX, true>::SMEM;
        return plan_one<T, TX, true, true>(per_sm);
    }
    smem = StGeom<T, TX, false>::SMEM;
    return forced ? plan_one<T, TX, false, true>(per_sm) : plan_one<T, TX, false, false>(per_sm);
}

template <class T>
static cudaError_t plan_t(int storage, const StepParams &P, bool thermal, void *const f[2], void *const g[2],
                          StagedPlan &sp) {
    sp = StagedPlan();
    int tx = 0;
    for (int c : {64, 32})
        if (P.nx % c == 0 && P.ny % (kStThreads / c) == 0) {
            tx = c;
            break;
        }
    if (tx == 0 || (P.nx * sizeof(T)) % 16 != 0 || (P.S * sizeof(T)) % 16 != 0 || !encode_fn() ||
        (!kStTmaStore && !P.idx32))
        return cudaSuccess;
    const int ty = kStThreads / tx, H = 16 / (int)sizeof(T);
    for (int b = 0; b < 2; b++) {
        if (!make_map(&sp.maps[b][0], storage, f[b], P, Q, tx, ty) ||
            !make_map(&sp.maps[b][1], storage, f[b], P, Q, tx + H, ty))
            return cudaSuccess;
        if (thermal) {
            if (!make_map(&sp.maps[b][2], storage, g[b], P, QT, tx, ty) ||
                !make_map(&sp.maps[b][3], storage, g[b], P, QT, tx + H, ty))
                return cudaSuccess;
        } else {
            sp.maps[b][2] = sp.maps[b][0];
            sp.maps[b][3] = sp.maps[b][1];
        }
    }
    int per_sm = 0, dev = 0, sms = 0;
    size_t smem = 0;
    const bool forced = P.forced != 0;
    cudaError_t e =
        tx == 64 ? plan_tx<T, 64>(thermal, forced, per_sm, smem) : plan_tx<T, 32>(thermal, forced, per_sm, smem);
    if (e != cudaSuccess) return e;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    if (per_sm < 1) return cudaSuccess;
    sp.tx = tx;
    sp.ty = ty;
    sp.tiles_x = P.nx / tx;
    sp.tiles_y = P.ny / ty;
    sp.ntiles = (long long)sp.tiles_x * sp.tiles_y * P.nz;
    // every block resident at once: blocks that had to wait for a free slot
    // would run all their tiles after the others
    sp.grid = (int)std::min<long long>(sp.ntiles, (long long)per_sm * sms);
    sp.smem = smem;
    sp.enabled = 1;
    return cudaSuccess;
}

cudaError_t plan_staged(int storage, bool thermal, const StepParams &P, void *const f[2], void *const g[2],
                        StagedPlan &sp) {
    switch (storage) {
    case 0: return plan_t<float>(storage, P, thermal, f, g, sp);
    case 1: return plan_t<__half>(storage, P, thermal, f, g, sp);
    case 2: return plan_t<__nv_bfloat16>(storage, P, thermal, f, g, sp);
    }
    return cudaErrorInvalidValue;
}

template <class T, int TX>
static void launch_tx(const LaunchArgs &a) {
    const StagedPlan &sp = *a.st;
    const CUtensorMap *mA = sp.maps[a.buf_a], *mB = sp.maps[1 - a.buf_a];
    const T *A = (const T *)a.A, *GA = (const T *)a.GA;
    if (a.thermal)
        k_step_st<T, TX, true, true><<<sp.grid, kStBlock, sp.smem, a.stream>>>(
            mA[0], mA[1], mB[0], mA[2], mA[3], mB[2], A, GA, (T *)a.B, (T *)a.GB, *a.P, a.ds, a.band, a.region, sp.tiles_x, sp.tiles_y,
            sp.ntiles);
    else if (a.P->forced)
        k_step_st<T, TX, false, true><<<sp.grid, kStBlock, sp.smem, a.stream>>>(
            mA[0], mA[1], mB[0], mA[2], mA[3], mB[2], A, GA, (T *)a.B, (T *)a.GB, *a.P, a.ds, a.band, a.region, sp.tiles_x, sp.tiles_y,
            sp.ntiles);
    else
        k_step_st<T, TX, false, false><<<sp.grid, kStBlock, sp.smem, a.stream>>>(
            mA[0], mA[1], mB[0], mA[2], mA[3], mB[2], A, GA, (T *)a.B, (T *)a.GB, *a.P, a.ds, a.band, a.region, sp.tiles_x, sp.tiles_y,
            sp.ntiles);
}

template <class T>
static void launch_t(const LaunchArgs &a) {
    if (a.st->tx == 64)
        launch_tx<T, 64>(a);
    else
        launch_tx<T, 32>(a);
}

cudaError_t launch_staged(int storage, const LaunchArgs &a) {
    switch (storage) {
    case 0: launch_t<float>(a); break;
    case 1: launch_t<__half>(a); break;
    case 2: launch_t<__nv_bfloat16>(a); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace lbmk
