// Ozaki-scheme split-precision block products on tcgen05 tensor cores
// (see bsg_ozaki.cuh for the arithmetic).
//
// k_ozgemm: persistent, one CTA per SM.
//   warp 0     producer: per step, bulk-copies the digit images of up to R
//              A blocks (one per row slot; a zero image where the screen
//              drops the pair) and of the shared B block into a stage of the
//              shared-memory ring (cp.async.bulk, mbarrier transaction count).
//   warp 1     MMA issuer (one thread): per k16 step and A digit i, one
//              tcgen05.mma D_i x [E_0..E_{nd-1-i}] into TMEM region i; a chain
//              of <= 512 k is committed to the epilogue.
//   warps 2-   epilogue, G groups of four warps (one TMEM lane quadrant per
//              warp, NP / G columns per group; G = 3 at 24 and 48 columns,
//              else 2): per chain, the exact regions R0 (integers), R1 (multiples
//              of 2^-8) and R2 (multiples of 2^-16) are added as integers into
//              an int64 accumulator, the lower-weight regions in FP32; once per
//              tile the two are combined (in integers up to 5 digits), scaled
//              by 2^(e_row + f_col - 14) and the output blocks written (GB300's
//              FP64 rate is far below its integer / FP32 rates).
// Every mbarrier wait is bounded (2 s); a timeout raises a flag that ends
// all roles and is returned as BSG_ERR_TIMEOUT.
#include <algorithm>
#include <atomic>
#include <tuple>
#include <mutex>

#include "bsg_ozaki.cuh"
#include "bsg_rik.cuh"
#include "bsg_tc.cuh"

namespace bsg {

using bf16 = __nv_bfloat16;

// zeros for masked slots: the A images of a pair of the largest steps
// (2 x 8 digits x 128 rows x 64 k; a run of masked slots may span both)
static __device__ __align__(128) bf16 g_oz_zero[2 * 8 * 128 * 64];

static void *oz_zero_image() {
    static std::mutex mu;
    static void *addr[64] = {};
    int dev = 0;
    BSG_CUDA(cudaGetDevice(&dev));
    BSG_REQUIRE(dev >= 0 && dev < 64, BSG_ERR_UNSUPPORTED, "device index out of range");
    std::lock_guard<std::mutex> lk(mu);
    if (!addr[dev]) BSG_CUDA(cudaGetSymbolAddress(&addr[dev], g_oz_zero));
    return addr[dev];
}

static int round_up(int x, int m) { return (x + m - 1) / m * m; }

// B rows of a stage: the nd stacked digit planes, rounded up to the MMA's
// N granularity of 16 (an MMA over an odd number of 8-row planes reads 8
// zero rows past the stack)
static uint32_t oz_b_rows(int nd, int np) { return (uint32_t)round_up(nd * np, 16); }
// bytes of one stage in shared memory: one step's A (128 rows) and B, or a
// pair's [A0 A1 B0 B1] with each A holding its R slots only.  The MMA reads
// 128 rows of A1 (a_stage bytes from its start), which run on into B0 and
// B1; where the slots hold fewer rows than B0 and B1 cover (8-row blocks: 64
// rows of slots) the stage is extended so that the read stays inside it.
static uint32_t oz_stage_bytes(const OzShape &sh) {
    const uint32_t b = oz_b_rows(sh.nd, sh.np) * sh.kp * 2u, a_stage = (uint32_t)sh.nd * 128u * sh.kp * 2u;
    if (!sh.pair) return a_stage + b;
    const uint32_t a_pack = (uint32_t)sh.R * sh.nd * sh.mp * sh.kp * 2u;
    return std::max(2u * a_pack + 2u * b, a_pack + a_stage);
}
constexpr uint32_t kOzSmemBudget = 200u * 1024u;
// room for the pipeline stages themselves: up to 224 KB of the 227 KB a CTA
// can have (the step prefetch and the barriers take the rest)
constexpr uint32_t kOzSmemStages = 224u * 1024u;

OzShape oz_shape(int bs_rows, int bs_k, int bs_cols, int nd) {
    OzShape s;
    s.nd = nd;
    s.mp = round_up(bs_rows, 8);
    s.np = round_up(bs_cols, 8);
    s.R = std::min(kOzMaxSlots, 128 / s.mp);
    // k rounded up to 8 leaves an odd number of 8-wide core columns: pair the
    // steps (no zero padding in k) where two stages of pairs fit
    s.kp = round_up(bs_k, 8);
    s.pair = (s.kp % 16 == 8) ? 1 : 0;
    if (s.pair && kOzSmemBudget / oz_stage_bytes(s) < 2) s.pair = 0;
    if (!s.pair) s.kp = round_up(bs_k, 16);
    s.F = s.pair ? 2 * std::max(1, 512 / (2 * s.kp)) : std::max(1, 512 / s.kp);
    return s;
}

int oz_default_digits(int requested, int bs_rows, int bs_k, int bs_cols) {
    if (requested) {
        const OzShape sh = oz_shape(bs_rows, bs_k, bs_cols, requested);
        BSG_REQUIRE(requested >= 2 && requested <= kOzMaxDigits, BSG_ERR_ARG, "Ozaki form: 2..8 digits");
        BSG_REQUIRE(kOzSmemBudget / oz_stage_bytes(sh) >= 2, BSG_ERR_UNSUPPORTED,
                    "Ozaki form: this digit count does not fit shared memory for the block size");
        return requested;
    }
    // 5 digits (~1e-11 relative per product) where two pipeline stages fit, else 4
    const OzShape s5 = oz_shape(bs_rows, bs_k, bs_cols, 5);
    return kOzSmemBudget / oz_stage_bytes(s5) >= 2 ? 5 : 4;
}

// Geometry of a run of tiles: an OzShape with its operand images.  A launch
// holds one; a launch over a batch of products of several block sizes holds
// one per block-size group, its tiles in group order: tiles below
// geo[0].tile_end have geometry 0, the next ones up to geo[1].tile_end
// geometry 1, and so on.
struct OzGeo {
    int mp, kp, np, R, nd, F;
    int pair;           // two steps per stage (OzShape::pair)
    int J;              // N-side sub-blocks of a B image (np / J rows each)
    uint32_t tx_bytes;  // bytes of one step's copies
    int S;                // pipeline stages of this geometry's tiles
    uint32_t stage_bytes; // their stride in the shared-memory ring
    uint32_t tile_end;
    const bf16 *a_img, *b_img;
};
constexpr int kOzMaxGeo = 8;

struct OzKParams {
    OzGeo geo[kOzMaxGeo];
    int n_geo;
    int S;                 // stage barriers: the most stages of any geometry
    uint32_t ring_bytes;   // the shared-memory ring: the largest S x stage_bytes of any geometry
    uint32_t chunk;        // consecutive tiles per CTA turn
    int nbuf;              // TMEM accumulator sets (2: the MMA fills one while the epilogue drains the other)
    uint32_t tmem_cols;    // columns of one accumulator set
    const bf16 *zero;
    double alpha;
    unsigned long long *prof;  // optional stall counters (kOzProf entries), null when not timing
};

// Shared-memory layout of one stage for a geometry (np = the tile's output
// columns).  One step: [A: 128 rows | B].  A pair: [A0 | A1 | B0 | B1] with
// each A holding only its R slots (a_pack bytes), so that the two steps'
// slot images sit back to back as they do in the A images when the image
// indices continue from one step to the next (one copy instead of two; a
// bulk copy's cost is mostly per copy).  The MMA still reads 128 rows of each
// A: rows past the R slots fall in the next region of the same stage (finite
// digits), and their accumulator rows are never stored.
struct OzLay {
    uint32_t a_stage;     // A: 128 rows x nd digits (M-side layout)
    uint32_t b_copy;      // bytes of one B digit stack
    uint32_t b_stage;     // its room in the stage (N rounded to 16)
    uint32_t slot_bytes;  // one slot's full digit image
    uint32_t a_pack;      // A bytes of one step
    uint32_t b_off;       // offset of B0 in the stage
    size_t slot_elems, b_img_elems;
};
__device__ __forceinline__ OzLay oz_lay(const OzGeo &g, int np) {
    OzLay L;
    L.a_stage = (uint32_t)g.nd * 128u * g.kp * 2u;
    L.b_copy = (uint32_t)g.nd * np * g.kp * 2u;
    L.b_stage = (uint32_t)((g.nd * np + 15) & ~15) * g.kp * 2u;
    L.slot_bytes = (uint32_t)g.nd * g.mp * g.kp * 2u;
    L.a_pack = g.pair ? (uint32_t)g.R * L.slot_bytes : L.a_stage;
    L.b_off = g.pair ? 2u * L.a_pack : L.a_stage;
    L.slot_elems = (size_t)g.nd * g.mp * g.kp;
    L.b_img_elems = (size_t)g.nd * np * g.kp;
    return L;
}
// geometry index of tile t
__device__ __forceinline__ int oz_geo_index(const OzGeo *geo, int n_geo, uint32_t t) {
    int i = 0;
    while (i + 1 < n_geo && t >= geo[i].tile_end) ++i;
    return i;
}

// stall counters (SM clock cycles summed over CTAs), read through bsg_ctx_gemm_stalls
enum OzProf {
    kProfMmaWaitFull,    // MMA issuer waiting for operand stages
    kProfMmaWaitTmem,    // MMA issuer waiting for a drained accumulator set
    kProfMmaTotal,       // MMA issuer lifetime
    kProfProdWaitEmpty,  // producer waiting for a free stage
    kProfEpiWaitFull,    // epilogue waiting for a finished chain
    kProfEpiDrain,       // epilogue reading TMEM and accumulating
    kProfEpiStore,       // epilogue scaling and writing output blocks
    kProfSteps,          // operand stages consumed by the MMA issuer
    kProfMmas,           // tcgen05.mma instructions issued
    kProfCopiedSteps,    // k steps copied by the producer (a pair stage holds two)
    kProfLivePairs,      // (live slot, copied N-side sub-block) pairs over those steps (a zero-image
                         // sub-block that rides along in a whole-image copy counts)
    kProfPairCapacity,   // slots x sub-blocks over those steps
    kOzProf
};
static_assert(kOzProf == 12, "the context keeps 12 GEMM counters");

// Warps: producer, MMA issuer, then the epilogue: four TMEM lane quadrants x
// G column groups.  Its per-element conversions and stores are integer
// instructions on the four schedulers, so where the columns split into three
// groups of whole 8-column loads (24 and 48 columns: the RI-K shapes) the
// epilogue has 12 warps, three per scheduler.  Registers: each of the SM's
// four partitions holds 16384, and a CTA's warps are spread over them
// round-robin, so the busiest partition's ceil(warps / 4) warps set the
// per-thread cap (14 warps: 128; 10 warps: 168).
template <int NP>
struct OzEpi {
    static constexpr int G = (NP == 24 || NP == 48) ? 3 : 2;
    static constexpr int warps = 2 + 4 * G;
    static constexpr int threads = 32 * warps;
    static constexpr int max_regs = (16384 / (32 * ((warps + 3) / 4))) / 8 * 8;
};

// Helpers of the epilogue's conversions.  FP64 arithmetic stays off its
// common path (GB300 runs FP64 at a small fraction of its integer rate); the
// float -> int64 and int64 -> double conversions are the hardware ones, one
// instruction each, where integer restatements are long dependent chains.
// v 2^e outside the fast paths (zero, subnormal or out-of-range results): an
// ordinary multiplication by the power of two, as volatile inline PTX so that
// the compiler branches around it instead of if-converting it (a warp's FP64
// multiply holds GB300's FP64 pipe for tens of clocks; an if-converted copy
// would run for every element)
__device__ __forceinline__ double oz_scale_pow2_slow(double v, int e) {
    const double sc = (e >= -1022 && e <= 1023) ? __longlong_as_double((long long)(e + 1023) << 52) : ldexp(1.0, e);
    double r;
    asm volatile("mul.rn.f64 %0, %1, %2;" : "=d"(r) : "d"(v), "d"(sc));
    return r;
}
// an FP32 value as a double (exact; zero and subnormal inputs take the
// hardware conversion)
__device__ __forceinline__ double oz_f32_to_f64(float f) {
    const uint32_t u = __float_as_uint(f);
    const uint32_t ex = (u >> 23) & 0xFFu;
    if (ex == 0u || ex == 0xFFu) {  // rare: kept out of the common path (see oz_scale_pow2_slow)
        double r;
        asm volatile("cvt.f64.f32 %0, %1;" : "=d"(r) : "f"(f));
        return r;
    }
    return __longlong_as_double((long long)(((unsigned long long)(u >> 31) << 63) |
                                            ((unsigned long long)(ex - 127u + 1023u) << 52) |
                                            ((unsigned long long)(u & 0x7FFFFFu) << 29)));
}
// v 2^e: the exponent field moves when the result stays a normal number
__device__ __forceinline__ double oz_scale_pow2(double v, int e) {
    const long long b = __double_as_longlong(v);
    const int ev = (int)((b >> 52) & 0x7FF);
    const int en = ev + e;
    if (ev != 0 && ev != 0x7FF && en > 0 && en < 0x7FF) return __longlong_as_double(b + ((long long)e << 52));
    return oz_scale_pow2_slow(v, e);
}

// Tile sequence of a CTA: chunks of `chunk` consecutive tiles, chunk
// blockIdx.x, then every gridDim.x-th chunk (tiles of one chunk share operand
// images, which then stay hot in L2 between them).  Every role walks the same
// sequence.
__device__ __forceinline__ uint32_t oz_first_tile(uint32_t chunk) { return blockIdx.x * chunk; }
__device__ __forceinline__ uint32_t oz_next_tile(uint32_t t, uint32_t chunk) {
    ++t;
    return (t % chunk) ? t : t + (gridDim.x - 1) * chunk;
}

// digits whose accumulator regions (nd x NP columns, + 8 for a rounded-up N)
// fit the 512 TMEM columns, and MMAs per k16 slice at that many digits
__host__ __device__ constexpr int oz_max_digits(int np) {
    return (512 - 8) / np < kOzMaxDigits ? (512 - 8) / np : kOzMaxDigits;
}
__host__ __device__ constexpr int oz_plan_entries(int nd, int planes) {
    int n = 0;
    for (int i = 0; i < nd; ++i) n += (nd - i + planes - 1) / planes;
    return n;
}

// MULTI: the launch holds several tile geometries (OzKParams::geo), each
// tile takes its own; NP is then the largest tile width.  Otherwise every
// tile has geometry 0, of width NP.
template <int NP, bool MULTI>
__global__ void __launch_bounds__(OzEpi<NP>::threads) __maxnreg__(OzEpi<NP>::max_regs)
    k_ozgemm(const OzTile *__restrict__ tiles, uint32_t n_tiles, const OzStep *__restrict__ steps,
             const __grid_constant__ OzKParams P, int *__restrict__ err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // The ring holds S stages of a geometry, each oz_stage_bytes of it (every
    // byte the MMAs read from a stage, also A1's 128 rows in pair mode).  A
    // multi-geometry launch changes S and the stride at a change of geometry
    // (the producer first waits for every stage to be released); a stage's
    // barriers keep their own phase across the change (bit s of phb).
    const OzLay L0 = oz_lay(P.geo[0], NP);  // the stage layout of a one-geometry launch
    OzStep *sstep = reinterpret_cast<OzStep *>(smem + (size_t)P.ring_bytes);  // 32 prefetched steps
    uint64_t *full = reinterpret_cast<uint64_t *>(sstep + 32);
    uint64_t *empty = full + P.S;
    uint64_t *tfull = empty + P.S;  // [2]
    uint64_t *tempty = tfull + 2;   // [2]
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(tempty + 2);
    volatile int *abort = reinterpret_cast<volatile int *>(tmem_slot + 1);
    OzGeo *sgeo = reinterpret_cast<OzGeo *>(tmem_slot + 4);  // MULTI: the geometry table
    const bool prof = P.prof != nullptr;
    // geometry of tile t and its stage layout
    auto geo_at = [&](uint32_t t) -> const OzGeo & {
        if constexpr (MULTI) return sgeo[oz_geo_index(sgeo, P.n_geo, t)];
        else return P.geo[0];
    };
    auto lay_of = [&](const OzGeo &g) -> OzLay {
        if constexpr (MULTI) return oz_lay(g, g.np);
        else return L0;
    };

    if (threadIdx.x == 0) {
        for (int s = 0; s < P.S; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(&tfull[b], 1);
            tc::mbar_init(&tempty[b], 4 * OzEpi<NP>::G);
        }
        *abort = 0;
        tc::fence_barrier_init();
    }
    if constexpr (MULTI) {
        if (threadIdx.x < (unsigned)P.n_geo) sgeo[threadIdx.x] = P.geo[threadIdx.x];
    }
    // rows past the last slot are never copied: keep them zero
    for (uint32_t i = threadIdx.x; i < P.ring_bytes / 16u; i += blockDim.x)
        reinterpret_cast<uint4 *>(smem)[i] = make_uint4(0, 0, 0, 0);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    if (warp == 1) {
        tc::tmem_alloc(tmem_slot, P.tmem_cols * P.nbuf);
        tc::tmem_relinquish();
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        // ---------------- producer ----------------
        uint32_t it = 0;  // stages filled
        unsigned long long w_empty = 0;
        // ring position; a one-geometry launch flips ph at every wrap, a
        // multi-geometry one keeps each stage's phase (bit s of phb) and the
        // stages ever filled
        uint32_t stage = 0, ph = 0, phb = 0, filled = 0;
        int cur_geo = -1;
        uint32_t n_stages = (uint32_t)P.geo[0].S, sbytes = P.geo[0].stage_bytes;
        unsigned long long n_copied = 0, n_live = 0, n_cap = 0;
        // the A slots of a stage: lane l < nA takes slot l % R of step l / R,
        // at sA + l * slot_bytes (a pair's second step follows the first).
        // Runs of consecutive images (or of zeros) go in one copy: a fully
        // live step is one A copy, and so is a fully live pair whose image
        // indices continue from the first step to the second
        auto copy_a = [&](const OzGeo &g, const OzLay &L, const OzStep &st0, const OzStep &st1, bool two, uint8_t *sA,
                          uint64_t *bar) {
            const uint32_t nA = two ? 2u * (uint32_t)g.R : (uint32_t)g.R;
            const uint32_t ai =
                lane < g.R ? st0.a[lane] : ((uint32_t)lane < nA ? st1.a[lane - g.R] : kOzNone);
            const uint32_t prev = __shfl_up_sync(0xffffffffu, ai, 1);
            const bool live = ai != kOzNone;
            const bool joins = lane > 0 && (live ? (prev != kOzNone && prev + 1u == ai) : prev == kOzNone);
            const uint32_t starts = __ballot_sync(0xffffffffu, (uint32_t)lane < nA && !joins) | (1u << nA);
            if ((uint32_t)lane < nA && !joins) {
                const int len = __ffs(starts & ~((2u << lane) - 1u)) - 1 - lane;
                const bf16 *src = live ? g.a_img + (size_t)ai * L.slot_elems : P.zero;
                tc::bulk_g2s(sA + lane * L.slot_bytes, src, (uint32_t)len * L.slot_bytes, bar);
            }
        };
        // one step's B digit stack into sB
        auto copy_b = [&](const OzGeo &g, const OzLay &L, const OzStep &st, uint8_t *sB, uint64_t *bar) {
            const uint32_t jfull = (1u << g.J) - 1u;
            if ((st.bmask & jfull) == jfull) {
                if (lane == 31) tc::bulk_g2s(sB, g.b_img + (size_t)st.b * L.b_img_elems, L.b_copy, bar);
            } else {
                // some N-side sub-blocks are screened out for this step: per
                // (sub-block, digit) chunk, the image's rows or zeros
                const int np = MULTI ? g.np : NP;
                const int npj = np / g.J, c = lane - 16;
                if (c >= 0 && c < g.J * g.nd) {
                    const int j = c / g.nd, i = c % g.nd;
                    const size_t off = ((size_t)i * np + (size_t)j * npj) * g.kp;
                    const bf16 *src =
                        ((st.bmask >> j) & 1u) ? g.b_img + (size_t)st.b * L.b_img_elems + off : P.zero;
                    tc::bulk_g2s(sB + off * 2, src, (uint32_t)npj * g.kp * 2u, bar);
                }
            }
        };
        auto count_step = [&](const OzGeo &g, const OzStep &st) {
            const bool live = lane < g.R && st.a[lane] != kOzNone;
            ++n_copied;
            n_cap += (unsigned long long)(g.R * g.J);
            n_live += (unsigned long long)__popc(__ballot_sync(0xffffffffu, live)) *
                      (unsigned long long)__popc(st.bmask & ((1u << g.J) - 1u));
        };
        bool pok = true;
        for (uint32_t t = oz_first_tile(P.chunk); t < n_tiles && pok && !*abort; t = oz_next_tile(t, P.chunk)) {
            const OzGeo &g = geo_at(t);
            const OzLay L = lay_of(g);
            const int gi = MULTI ? oz_geo_index(sgeo, P.n_geo, t) : 0;
            if (MULTI && gi != cur_geo) {
                // a new geometry: every filled stage released before the ring is laid out anew
                if (cur_geo >= 0 && lane == 0) {
                    for (int s2 = 0; s2 < P.S && pok; ++s2)
                        if ((filled >> s2) & 1u) pok = tc::mbar_wait_sleep(&empty[s2], ((phb >> s2) & 1u) ^ 1u, abort);
                }
                pok = __shfl_sync(0xffffffffu, pok ? 1 : 0, 0) != 0;
                if (!pok) break;
                cur_geo = gi;
                stage = 0;
                n_stages = (uint32_t)g.S;
                sbytes = g.stage_bytes;
            }
            const uint32_t jfull = (1u << g.J) - 1u, kstep = g.pair ? 2u : 1u;
            const uint32_t s0 = tiles[t].s0, ns = tiles[t].ns;
            for (uint32_t k = 0; k < ns; k += kstep, ++it) {
                if ((k & 31u) == 0) {
                    // the warp loads the next 32 step descriptors at once (a
                    // pair never crosses a batch: k is even in pair mode)
                    __syncwarp();
                    if (k + lane < ns) sstep[lane] = steps[s0 + k + lane];
                    __syncwarp();
                }
                // one lane waits, the warp follows its verdict (keeps the warp converged)
                int okw = 1;
                if (lane == 0) {
                    const long long c0 = prof ? clock64() : 0;
                    const uint32_t par = MULTI ? ((phb >> stage) & 1u) ^ 1u : ph ^ 1u;
                    okw = tc::mbar_wait_sleep(&empty[stage], par, abort) ? 1 : 0;
                    if (prof) w_empty += clock64() - c0;
                }
                if (!__shfl_sync(0xffffffffu, okw, 0)) break;
                uint8_t *sA = smem + (size_t)stage * sbytes;
                uint8_t *sB = sA + L.b_off;
                const bool two = g.pair && k + 1 < ns;
                // a lone last step of a pair stage gets a zero B in the second
                // half: the k16 slice that straddles into it then adds nothing
                // (its A half holds earlier digits or zeros, always finite)
                const uint32_t tx = two ? 2u * g.tx_bytes : (g.pair ? g.tx_bytes + L.b_copy : g.tx_bytes);
                if (lane == 0) tc::mbar_arrive_expect_tx(&full[stage], tx);
                __syncwarp();
                const OzStep &st0 = sstep[k & 31u], &st1 = sstep[(k + 1) & 31u];
                if (prof) {
                    count_step(g, st0);
                    if (two) count_step(g, st1);
                }
                copy_a(g, L, st0, st1, two, sA, &full[stage]);
                if (two && L.b_stage == L.b_copy && (st0.bmask & jfull) == jfull && (st1.bmask & jfull) == jfull &&
                    st1.b == st0.b + 1u) {
                    // both steps' full B stacks, consecutive in the B images: one copy
                    if (lane == 31)
                        tc::bulk_g2s(sB, g.b_img + (size_t)st0.b * L.b_img_elems, 2u * L.b_copy, &full[stage]);
                } else {
                    copy_b(g, L, st0, sB, &full[stage]);
                    if (two)
                        copy_b(g, L, st1, sB + L.b_stage, &full[stage]);
                    else if (g.pair && lane == 31)
                        tc::bulk_g2s(sB + L.b_stage, P.zero, L.b_copy, &full[stage]);
                }
                if constexpr (MULTI) {
                    phb ^= 1u << stage;
                    filled |= 1u << stage;
                    if (++stage == n_stages) stage = 0;
                } else if (++stage == (uint32_t)P.S) {
                    stage = 0;
                    ph ^= 1u;
                }
            }
        }
        // let the copies in flight land before the CTA can exit: the last
        // fill of every stage
        if (lane == 0) {
            if constexpr (MULTI) {
                for (int s2 = 0; s2 < P.S; ++s2)
                    if ((filled >> s2) & 1u) tc::mbar_wait(&full[s2], ((phb >> s2) & 1u) ^ 1u, abort);
            } else {
                const uint32_t first = it > (uint32_t)P.S ? it - P.S : 0;
                for (uint32_t j = first; j < it; ++j) tc::mbar_wait(&full[j % P.S], (j / P.S) & 1u, abort);
            }
            if (prof) {
                atomicAdd(&P.prof[kProfProdWaitEmpty], w_empty);
                atomicAdd(&P.prof[kProfCopiedSteps], n_copied);
                atomicAdd(&P.prof[kProfLivePairs], n_live);
                atomicAdd(&P.prof[kProfPairCapacity], n_cap);
            }
        }
        __syncwarp();
    } else if (warp == 1) {
        // ---------------- MMA issuer ----------------
        if (lane == 0) {
            const long long t_start = prof ? clock64() : 0;
            unsigned long long w_full = 0, w_tmem = 0, n_mma = 0;
            uint32_t it = 0, ch = 0, stage = 0, ph = 0, phb = 0;  // phb: per-stage phases (multi-geometry)
            // MMA plan of one k16 slice for a geometry: per A digit i, D_i x
            // [E_j0 .. E_j1) stacked along N (N <= 256, rounded up to 16: the
            // extra columns land past the last region) into TMEM region i + j0.
            // Entry: x = TMEM column | (i == 0) << 16, y / z = A / B descriptor
            // address offsets (16-byte units), w = instruction descriptor.  The
            // plan is held in registers (the loops below are unrolled); a
            // multi-geometry launch rebuilds it when the geometry changes.
            constexpr int kMaxPlanes = 256 / NP;  // B planes one MMA can take at width NP
            constexpr int kMaxPlan = oz_plan_entries(oz_max_digits(NP), kMaxPlanes);
            uint32_t pd[kMaxPlan], pa[kMaxPlan], pb[kMaxPlan], pi[kMaxPlan];
            int n_plan = 0;
            uint64_t a_desc0 = 0, b_desc0 = 0, a_descx = 0, b_descx = 0;
            uint32_t ncol = 0, cF = 1, ckstep = 1, ca_pack = 0, cb_stage = 0;
            int cpair = 0, ckp = 0;
            auto setup = [&](const OzGeo &g, const OzLay &L) {
                const int np = MULTI ? g.np : NP;
                const int planes = MULTI ? 256 / np : kMaxPlanes;
                // 8-row groups: nd*kp*16 bytes apart on the M side (digits interleaved), kp*16 on the N side
                a_desc0 = tc::smem_desc(tc::smem_u32(smem), 128u, (uint32_t)g.nd * g.kp * 16u);
                b_desc0 = tc::smem_desc(tc::smem_u32(smem + L.b_off), 128u, (uint32_t)g.kp * 16u);
                // pair mode: the slice that straddles the two steps starts at the
                // first step's last core column and finds its second one (column 0
                // of the second step, a_pack / b_stage further on) one leading byte
                // offset further
                ncol = (uint32_t)g.kp / 8u;  // core columns per step
                const uint32_t lbo_xa = L.a_pack - (ncol - 1u) * 128u, lbo_xb = L.b_stage - (ncol - 1u) * 128u;
                a_descx = tc::smem_desc(tc::smem_u32(smem), lbo_xa, (uint32_t)g.nd * g.kp * 16u);
                b_descx = tc::smem_desc(tc::smem_u32(smem + L.b_off), lbo_xb, (uint32_t)g.kp * 16u);
                cF = (uint32_t)g.F;
                cpair = g.pair;
                ckp = g.kp;
                ckstep = g.pair ? 2u : 1u;
                ca_pack = L.a_pack;
                cb_stage = L.b_stage;
                n_plan = 0;
#pragma unroll
                for (int e = 0; e < kMaxPlan; ++e) pd[e] = pa[e] = pb[e] = pi[e] = 0;
                for (int i = 0; i < g.nd; ++i)
                    for (int j0 = 0; j0 < g.nd - i; j0 += planes) {
                        const int j1 = min(g.nd - i, j0 + planes);
#pragma unroll
                        for (int e = 0; e < kMaxPlan; ++e)
                            if (e == n_plan) {
                                pd[e] = (uint32_t)((i + j0) * np) | (i == 0 ? 1u << 16 : 0u);
                                pa[e] = ((uint32_t)i * g.kp * 16u) >> 4;
                                pb[e] = ((uint32_t)j0 * np * g.kp * 2u) >> 4;
                                pi[e] = tc::idesc_bf16_f32(128u, (uint32_t)(((j1 - j0) * np + 15) & ~15));
                            }
                        ++n_plan;
                    }
            };
            setup(P.geo[0], MULTI ? oz_lay(P.geo[0], P.geo[0].np) : L0);  // L0 is laid out for width NP
            int cur_geo = 0;
            uint32_t n_stages = (uint32_t)P.geo[0].S, sbytes16 = P.geo[0].stage_bytes >> 4;
            bool ok = true;
            // the tile / chain / stage walk; issue(soff, k, ns, first, dbase)
            // issues one stage's MMAs
            auto mma_loop = [&](auto &&issue) {
                for (uint32_t t = oz_first_tile(P.chunk); t < n_tiles && ok; t = oz_next_tile(t, P.chunk)) {
                    if constexpr (MULTI) {
                        const int gi = oz_geo_index(sgeo, P.n_geo, t);
                        if (gi != cur_geo) {
                            cur_geo = gi;
                            setup(sgeo[gi], oz_lay(sgeo[gi], sgeo[gi].np));
                            stage = 0;  // the producer lays the ring out anew
                            n_stages = (uint32_t)sgeo[gi].S;
                            sbytes16 = sgeo[gi].stage_bytes >> 4;
                        }
                    }
                    const uint32_t ns = tiles[t].ns;
                    const uint32_t nch = (ns + cF - 1) / cF;
                    for (uint32_t c = 0; c < nch && ok; ++c, ++ch) {
                        const uint32_t buf = P.nbuf == 2 ? (ch & 1u) : 0u, use = P.nbuf == 2 ? ch >> 1 : ch;
                        long long c0 = prof ? clock64() : 0;
                        if (!tc::mbar_wait(&tempty[buf], (use & 1u) ^ 1u, abort)) {
                            ok = false;
                            break;
                        }
                        if (prof) w_tmem += clock64() - c0;
                        tc::tc_fence_after();
                        const uint32_t dbase = tmem + buf * P.tmem_cols;
                        const uint32_t kend = min(ns, (c + 1) * cF);
                        for (uint32_t k = c * cF; k < kend; k += ckstep, ++it) {
                            c0 = prof ? clock64() : 0;
                            if (!tc::mbar_wait(&full[stage], MULTI ? (phb >> stage) & 1u : ph, abort)) {
                                ok = false;
                                break;
                            }
                            if (prof) w_full += clock64() - c0;
                            tc::tc_fence_after();
                            const uint32_t soff = stage * (MULTI ? sbytes16 : P.geo[0].stage_bytes >> 4);
                            // the first MMA of a chain (digit 0, which spans every TMEM
                            // region) overwrites the accumulator
                            issue(soff, k, ns, (k == c * cF) ? 1u : 0u, dbase);
                            tc::mma_commit(&empty[stage]);
                            if constexpr (MULTI) {
                                phb ^= 1u << stage;
                                if (++stage == n_stages) stage = 0;
                            } else if (++stage == (uint32_t)P.S) {
                                stage = 0;
                                ph ^= 1u;
                            }
                        }
                        if (!ok) break;
                        tc::mma_commit(&tfull[buf]);
                    }
                }
            };
            // any shape: the plan computed above, slices per stage at run time
            auto issue_generic = [&](uint32_t soff, uint32_t k, uint32_t ns, uint32_t first, uint32_t dbase) {
                // k16 slices of this stage: kp / 16 of one step, or, for a
                // pair, the ncol (odd) slices over both halves' 2 ncol core
                // columns -- of a lone last step only those touching its half
                const uint32_t nq = !cpair ? (uint32_t)ckp / 16u : (k + 1 < ns ? ncol : (ncol + 1u) / 2u);
                // slice descriptors of this stage
                uint64_t aqs[8], bqs[8];
#pragma unroll
                for (uint32_t q = 0; q < 8; ++q) {
                    uint64_t aq = 0, bq = 0;
                    if (q < nq) {
                        if (!cpair) {
                            aq = a_desc0 + soff + q * 16u;
                            bq = b_desc0 + soff + q * 16u;
                        } else {
                            const uint32_t g = 2u * q;  // first core column of the slice
                            if (g + 1u < ncol) {        // both in the first half
                                aq = a_desc0 + soff + g * 8u;
                                bq = b_desc0 + soff + g * 8u;
                            } else if (g + 1u == ncol) {  // straddles the halves
                                aq = a_descx + soff + g * 8u;
                                bq = b_descx + soff + g * 8u;
                            } else {  // both in the second step
                                aq = a_desc0 + soff + ((ca_pack + (g - ncol) * 128u) >> 4);
                                bq = b_desc0 + soff + ((cb_stage + (g - ncol) * 128u) >> 4);
                            }
                        }
                    }
                    aqs[q] = aq;
                    bqs[q] = bq;
                }
                // digit by digit, each over the stage's k16 slices: consecutive
                // MMAs accumulate into the same TMEM columns (a k chain), and
                // the first MMA of a chain (digit 0, which spans every region)
                // overwrites the accumulator
#pragma unroll
                for (int e = 0; e < kMaxPlan; ++e) {
                    if (e >= n_plan) break;
                    const uint32_t dt = dbase + (pd[e] & 0xFFFFu);
#pragma unroll
                    for (uint32_t q = 0; q < 8; ++q) {
                        if (q >= nq) break;
                        const uint32_t ac = (first && q == 0 && (pd[e] >> 16)) ? 0u : 1u;
                        tc::mma_bf16(dt, aqs[q] + pa[e], bqs[q] + pb[e], pi[e], ac);
                    }
                }
                if (prof) n_mma += (unsigned long long)n_plan * nq;
            };
            // blocks of 24 in step pairs, 5 digits, two N-side blocks (every
            // product of the RI-K step on 24-wide blocks): each descriptor is a
            // fixed offset from the stage's three A and three B slice
            // descriptors (only their low words depend on the stage) and the
            // MMA sequence is unrolled at compile time -- the single issuing
            // thread's instruction latency otherwise paces the tensor core
            auto issue_fixed = [&](uint32_t soff, uint32_t k, uint32_t ns, uint32_t first, uint32_t dbase) {
                constexpr uint32_t KP = 24, ND = 5;
                const uint32_t a_hi = (uint32_t)(a_desc0 >> 32), b_hi = (uint32_t)(b_desc0 >> 32);
                // the second step's core column 1
                const uint32_t ha2 = (L0.a_pack + 128u) >> 4, hb2 = (L0.b_stage + 128u) >> 4;
                const uint32_t a0 = (uint32_t)a_desc0 + soff, ax = (uint32_t)a_descx + soff + 16u, a2 = a0 + ha2;
                const uint32_t b0 = (uint32_t)b_desc0 + soff, bx = (uint32_t)b_descx + soff + 16u, b2 = b0 + hb2;
                const bool three = k + 1 < ns;  // a lone last step: the first two slices
                auto d64 = [](uint32_t lo, uint32_t hi) { return ((uint64_t)hi << 32) | lo; };
#pragma unroll
                for (uint32_t i = 0; i < ND; ++i) {
                    const uint32_t dt = dbase + i * (uint32_t)NP, pa = i * KP;
                    const uint32_t id = tc::idesc_bf16_f32(128u, ((ND - i) * (uint32_t)NP + 15u) & ~15u);
                    tc::mma_bf16(dt, d64(a0 + pa, a_hi), d64(b0, b_hi), id, (first && i == 0) ? 0u : 1u);
                    tc::mma_bf16(dt, d64(ax + pa, a_hi), d64(bx, b_hi), id, 1u);
                    if (three) tc::mma_bf16(dt, d64(a2 + pa, a_hi), d64(b2, b_hi), id, 1u);
                }
                if (prof) n_mma += three ? 3u * ND : 2u * ND;
            };
            if constexpr (NP == 48 && !MULTI) {
                if (P.geo[0].nd == 5 && P.geo[0].pair && P.geo[0].kp == 24 && n_plan == 5)
                    mma_loop(issue_fixed);
                else
                    mma_loop(issue_generic);
            } else {
                mma_loop(issue_generic);
            }
            if (prof) {
                atomicAdd(&P.prof[kProfMmaWaitFull], w_full);
                atomicAdd(&P.prof[kProfMmaWaitTmem], w_tmem);
                atomicAdd(&P.prof[kProfMmaTotal], (unsigned long long)(clock64() - t_start));
                atomicAdd(&P.prof[kProfSteps], (unsigned long long)it);
                atomicAdd(&P.prof[kProfMmas], n_mma);
            }
        }
        __syncwarp();
    } else {
        // ---------------- epilogue ----------------
        constexpr int NPH = NP / OzEpi<NP>::G;                           // columns per epilogue group
        constexpr int CH = (NPH % 8 == 0) ? 8 : 4;                       // TMEM columns per load
        static_assert(NPH % CH == 0, "a group's columns are whole TMEM loads");
        const int q = warp & 3;
        const int grp = (warp - 2) >> 2;
        const int m = q * 32 + lane;
        const uint32_t lane_off = (uint32_t)(q * 32) << 16;
        unsigned long long w_full = 0, t_drain = 0, t_store = 0;
        uint32_t ch = 0;
        bool ok = true;
        for (uint32_t t = oz_first_tile(P.chunk); t < n_tiles && ok; t = oz_next_tile(t, P.chunk)) {
            const OzGeo &g = geo_at(t);
            const int np = MULTI ? g.np : NP;  // TMEM columns per weight region
            // this group's columns: NP / G, or (a narrower geometry of a
            // multi-geometry launch) its width's share in whole TMEM loads
            const int npg = MULTI ? (np / OzEpi<NP>::G + CH - 1) / CH * CH : NPH;
            const int cbase = grp * npg;
            const OzTile &T = tiles[t];
            const uint32_t ns = T.ns;
            const uint32_t nch = (ns + g.F - 1) / g.F;
            long long hi[NPH];  // R0 + R1 + R2 in units of 2^-16
            float lo[NPH];      // R3 + R4 + ...
#pragma unroll
            for (int c = 0; c < NPH; ++c) {
                hi[c] = 0;
                lo[c] = 0.f;
            }
            for (uint32_t c = 0; c < nch; ++c, ++ch) {
                const uint32_t buf = P.nbuf == 2 ? (ch & 1u) : 0u, use = P.nbuf == 2 ? ch >> 1 : ch;
                long long c0 = prof ? clock64() : 0;
                if (!tc::mbar_wait_sleep(&tfull[buf], use & 1u, abort)) {
                    ok = false;
                    break;
                }
                tc::tc_fence_after();
                long long c1 = prof ? clock64() : 0;
                if (prof) w_full += c1 - c0;
                const uint32_t lane_addr = tmem + buf * P.tmem_cols + lane_off;
#pragma unroll
                for (int c0 = 0; c0 < NPH; c0 += CH) {
                    if (MULTI && c0 >= npg) break;
                    float v0[CH], v1[CH], v2[CH];
                    tc::tmem_ldn<CH>(lane_addr + (uint32_t)(cbase + c0), v0);
                    tc::tmem_ldn<CH>(lane_addr + (uint32_t)(np + cbase + c0), v1);
                    if (g.nd > 2) tc::tmem_ldn<CH>(lane_addr + (uint32_t)(2 * np + cbase + c0), v2);
                    tc::tmem_wait_ld();
                    // R0 is an integer < 2^24 and R1 a multiple of 2^-8 below 2^16: both
                    // exact in the FP32 accumulator.  R2 is a multiple of 2^-16 and exact
                    // while its partial sums stay below 2^8 (else rounded once here).
#pragma unroll
                    for (int j = 0; j < CH; ++j) {
                        long long h = ((long long)__float2int_rn(v0[j]) << 16) +
                                      ((long long)__float2int_rn(v1[j] * 256.f) << 8);
                        if (g.nd > 2) h += (long long)__float2int_rn(v2[j] * 65536.f);
                        hi[c0 + j] += h;
                    }
                    for (int w = 3; w < g.nd; ++w) {
                        float v[CH];
                        tc::tmem_ldn<CH>(lane_addr + (uint32_t)(w * np + cbase + c0), v);
                        tc::tmem_wait_ld();
#pragma unroll
                        for (int j = 0; j < CH; ++j) lo[c0 + j] += v[j];
                    }
                }
                tc::tc_fence_before();
                __syncwarp();
                if (lane == 0) tc::mbar_arrive(&tempty[buf]);
                if (prof) t_drain += clock64() - c1;
            }
            if (!ok) break;
            const long long c2 = prof ? clock64() : 0;
            const int s = m / g.mp, r = m % g.mp;
            if (s < g.R && T.c[s] != nullptr && r < T.rows[s]) {
                // value = alpha * (hi 2^-16 + lo) 2^(e_row + f_col - 14), formed as
                // (hi + lo 2^16) 2^(e_row + f_col - 30): the same rounding (scaling
                // by powers of two is exact), the power of two built from its bits
                const int er = T.rexp[s][r] - 30;
                double *cp = T.c[s];
                const int ldc = T.ldc[s];
                const bool fresh = (T.fresh_mask >> s) & 1u;
                const bool unit = P.alpha == 1.0;
                // sub-blocks stored apart (J <= 2 and G >= 2, so a group's NP / G
                // columns cross at most one sub-block boundary)
                const int tcols = T.cols, tsub = T.sub_cols, tcexp_sub = T.cexp_sub, ttrans = T.trans;
                const long long tsub_stride = T.sub_stride;
                const int *tcexp = T.cexp;
                const bool subm = tsub != 0;
                const int npj = np / g.J, js0 = cbase / npj;
                // every column's exponent loaded before the first store (the stores
                // could alias the exponent array, which would serialize the loads)
                int cex[NPH];
#pragma unroll
                for (int j = 0; j < NPH; ++j) {
                    const int c = cbase + j;
                    int cc = c, js = 0;
                    if (subm) {
                        js = c >= (js0 + 1) * npj ? js0 + 1 : js0;
                        cc = c - js * npj;
                    }
                    cex[j] = (c < tcols && (!subm || cc < tsub)) ? tcexp[subm ? js * tcexp_sub + cc : c] : 0;
                }
                // every output of the group, its value from total(j) scaled by
                // 2^(er + de + cex): one loop per way of forming the total, so
                // that no element pays for both
                auto store_all = [&](auto &&value, int de) {
                    // column j of this group: output address (null = not stored) and value
                    auto col_out = [&](int j, double *&dst) -> double {
                        const int c = cbase + j;
                        int cc = c, js = 0;
                        if (subm) {
                            js = c >= (js0 + 1) * npj ? js0 + 1 : js0;
                            cc = c - js * npj;
                        }
                        dst = nullptr;
                        if (!(c < tcols && (!subm || cc < tsub))) return 0.0;
                        const double out = value(j, er + de + cex[j]);
                        double *base = subm ? cp + js * tsub_stride : cp;
                        dst = ttrans ? base + cc + (size_t)r * ldc : base + r + (size_t)cc * ldc;
                        return out;
                    };
#pragma unroll
                    for (int j = 0; j < NPH; j += 2) {
                        if (MULTI && j >= npg) break;
                        double *d0, *d1;
                        const double o0 = col_out(j, d0), o1 = col_out(j + 1, d1);
                        // a transposed tile's row is contiguous in the output: pairs of
                        // columns go as one 16-byte store when adjacent and aligned
                        if (fresh && d0 && d1 == d0 + 1 && ((reinterpret_cast<uintptr_t>(d0) & 15u) == 0u)) {
                            *reinterpret_cast<double2 *>(d0) = make_double2(o0, o1);
                        } else {
                            if (d0) *d0 = fresh ? o0 : __dadd_rn(*d0, o0);
                            if (d1) *d1 = fresh ? o1 : __dadd_rn(*d1, o1);
                        }
                    }
                };
                // alpha (1 on every RI-K product) multiplies in a loop of its own,
                // so that the common case carries no FP64 multiply
                auto store_scaled = [&](auto &&value, int de) {
                    if (unit)
                        store_all(value, de);
                    else
                        store_all([&](int j, int e) { return __dmul_rn(P.alpha, value(j, e)); }, de);
                };
                if (g.nd <= 5 && nch < 256) {
                    // up to 5 digits lo holds weights 3 and 4, multiples of 2^-32,
                    // so lo 2^32 is an integer (below 2^34) and hi 2^16 + lo 2^32
                    // the exact sum in units of 2^-32 (hi < 2^39 per chain of <= 512
                    // k, so below 2^63 for < 256 chains): one rounding to double (the
                    // hardware int64 conversion, round to nearest even: the same as the
                    // FP64 add below makes), then the power of two put into the
                    // exponent field.  The conversion is one instruction per element;
                    // the same rounding done with integer operations is a long
                    // dependent chain that kept the epilogue waiting (occ products
                    // 18.9 -> 18.2 ms with the conversion)
                    store_scaled([&](int j, int e) {
                        return oz_scale_pow2(__ll2double_rn(hi[j] * 65536ll + __float2ll_rn(lo[j] * 4294967296.f)), e);
                    }, -16);
                } else {
                    // both terms are exact doubles (|hi| < 2^53, lo 2^16 an FP32
                    // value): one FP64 add rounds, and the power of two goes into the
                    // exponent field
                    store_scaled([&](int j, int e) {
                        return oz_scale_pow2(__dadd_rn(__ll2double_rn(hi[j]), oz_f32_to_f64(lo[j] * 65536.f)), e);
                    }, 0);
                }
                if (fresh && r == 0 && grp == 0 && T.cnorm[s]) *T.cnorm[s] = 0.0;
            }
            if (prof) t_store += clock64() - c2;
        }
        if (prof && lane == 0) {
            atomicAdd(&P.prof[kProfEpiWaitFull], w_full);
            atomicAdd(&P.prof[kProfEpiDrain], t_drain);
            atomicAdd(&P.prof[kProfEpiStore], t_store);
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 1) tc::tmem_dealloc(tmem, P.tmem_cols * P.nbuf);
    if (threadIdx.x == 0 && *abort) atomicExch(err, 1);
}

// TMEM columns the MMA plan of a geometry writes (per A digit i, planes
// j0..j1 stacked from column (i + j0) np, N rounded up to 16), with the
// MMA's planes per instruction for tile width np_max
static uint32_t oz_tmem_extent(int nd, int np, int np_max) {
    const int planes = 256 / np_max;
    uint32_t ext = 0;
    for (int i = 0; i < nd; ++i)
        for (int j0 = 0; j0 < nd - i; j0 += planes) {
            const int j1 = std::min(nd - i, j0 + planes);
            ext = std::max(ext, (uint32_t)((i + j0) * np + (((j1 - j0) * np + 15) & ~15)));
        }
    return ext;
}

// One launch over the tiles of one or several geometries (MULTI: each run of
// tiles has its own shape and images; the kernel is instantiated for the
// largest width NP, and a narrower geometry's MMAs take 256 / np planes).
template <int NP, bool MULTI>
static void launch_oz(bsg_ctx ctx, const std::vector<OzRun> &runs, const OzTile *tiles, size_t n_tiles,
                      const OzStep *steps, double alpha, int *err, unsigned long long *prof, uint32_t chunk,
                      cudaStream_t s) {
    BSG_REQUIRE(!runs.empty() && runs.size() <= (size_t)kOzMaxGeo && (MULTI || runs.size() == 1), BSG_ERR_UNSUPPORTED,
                "Ozaki launch: tile geometries");
    OzKParams P;
    P.chunk = chunk;
    P.n_geo = (int)runs.size();
    P.alpha = alpha;
    P.prof = prof;
    P.zero = static_cast<const bf16 *>(oz_zero_image());
    uint32_t ring = 0, cols = 0;
    int S = 0;
    constexpr int kMaxPlan = oz_plan_entries(oz_max_digits(NP), 256 / NP);
    for (size_t i = 0; i < runs.size(); ++i) {
        const OzShape &sh = runs[i].sh;
        const int np = MULTI ? sh.np : NP;
        BSG_REQUIRE(np == sh.np && np <= NP, BSG_ERR_UNSUPPORTED, "Ozaki launch: tile width");
        BSG_REQUIRE(sh.J >= 1 && sh.J * sh.nd <= 16 && np % sh.J == 0 && (np / sh.J) % 8 == 0, BSG_ERR_UNSUPPORTED,
                    "Ozaki tile: N-side sub-blocks");
        BSG_REQUIRE(!sh.pair || (sh.F % 2 == 0 && sh.kp % 16 == 8), BSG_ERR_UNSUPPORTED, "Ozaki tile: step pairs");
        BSG_REQUIRE(oz_plan_entries(sh.nd, 256 / np) <= kMaxPlan, BSG_ERR_UNSUPPORTED, "Ozaki tile: MMA plan");
        BSG_REQUIRE(i == 0 || runs[i].tile_end >= runs[i - 1].tile_end, BSG_ERR_ARG, "Ozaki launch: tile runs");
        OzGeo &g = P.geo[i];
        g.mp = sh.mp;
        g.kp = sh.kp;
        g.np = np;
        g.R = sh.R;
        g.nd = sh.nd;
        g.F = sh.F;
        g.pair = sh.pair;
        g.J = sh.J;
        g.tx_bytes = (uint32_t)sh.R * sh.nd * sh.mp * sh.kp * 2u + (uint32_t)sh.nd * np * sh.kp * 2u;
        g.tile_end = (uint32_t)runs[i].tile_end;
        g.a_img = runs[i].a_img;
        g.b_img = runs[i].b_img;
        {  // every byte an MMA reads lies inside the stage: A0/A1 128 rows each, B0/B1
            const uint32_t a_stage = (uint32_t)sh.nd * 128u * sh.kp * 2u, b_st = oz_b_rows(sh.nd, np) * sh.kp * 2u;
            const uint32_t a_pack = sh.pair ? (uint32_t)sh.R * sh.nd * sh.mp * sh.kp * 2u : a_stage;
            const uint32_t b_off = sh.pair ? 2u * a_pack : a_stage;
            const uint32_t reach = std::max((sh.pair ? a_pack : 0u) + a_stage, b_off + (sh.pair ? 2u : 1u) * b_st);
            BSG_REQUIRE(reach <= oz_stage_bytes(sh), BSG_ERR_UNSUPPORTED, "Ozaki tile: stage layout");
        }
        g.stage_bytes = oz_stage_bytes(sh);
        g.S = (int)std::min<uint32_t>(sh.S > 0 ? (uint32_t)sh.S : 4u, kOzSmemStages / g.stage_bytes);
        BSG_REQUIRE(g.S >= 2, BSG_ERR_UNSUPPORTED, "Ozaki tile does not fit shared memory");
        ring = std::max(ring, (uint32_t)g.S * g.stage_bytes);
        S = std::max(S, g.S);
        // the columns the MMAs write; the epilogue reads NP / G columns past
        // each region's start
        cols = std::max(cols, oz_tmem_extent(sh.nd, np, np));
        if (MULTI) cols = std::max(cols, (uint32_t)((sh.nd - 1) * np + NP));
    }
    BSG_REQUIRE(runs.back().tile_end == n_tiles, BSG_ERR_ARG, "Ozaki launch: tile runs");
    P.ring_bytes = ring;
    P.S = S;
    uint32_t tcols = 32;
    while (tcols < cols) tcols <<= 1;
    P.tmem_cols = tcols;
    P.nbuf = tcols <= 256 ? 2 : 1;
    BSG_REQUIRE(tcols <= 512, BSG_ERR_UNSUPPORTED, "Ozaki form: digits x padded block columns exceed TMEM");
    const size_t smem = (size_t)ring + 32 * sizeof(OzStep) + (2 * P.S + 4) * 8 + 16 +
                        (MULTI ? kOzMaxGeo * sizeof(OzGeo) : 0);
    {  // raise the shared-memory limit only when needed (never inside a graph capture)
        static std::atomic<int> set_to[64];
        int dev = 0;
        BSG_CUDA(cudaGetDevice(&dev));
        if (dev < 0 || dev >= 64 || (int)smem > set_to[dev].load()) {
            BSG_CUDA(cudaFuncSetAttribute(k_ozgemm<NP, MULTI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            if (dev >= 0 && dev < 64) set_to[dev].store((int)smem);
        }
    }
    const int sms = std::max(1, ctx->sm_count - ctx->oz_sm_reserve);
    const unsigned grid = (unsigned)std::min<size_t>(ceil_div(n_tiles, (size_t)chunk), (size_t)sms);
    BSG_REQUIRE(n_tiles + (size_t)grid * chunk < 0xffffffffull, BSG_ERR_UNSUPPORTED, "too many Ozaki tiles");
    k_ozgemm<NP, MULTI><<<grid, OzEpi<NP>::threads, smem, s>>>(tiles, (uint32_t)n_tiles, steps, P, err);
    ctx->note_launch();
    ctx->check_launch("ozaki gemm");
}

// one launch of the given runs; in timing mode with CUDA events around it,
// the kernel's stall counters and the useful multiply-adds (d_macs) read back
static void oz_launch_timed(bsg_ctx ctx, const std::vector<OzRun> &runs, const OzTile *d_tiles, size_t n_tiles,
                            const OzStep *d_steps, double alpha, cudaStream_t s, const unsigned long long *d_macs,
                            uint32_t chunk) {
    BSG_REQUIRE(chunk >= 1, BSG_ERR_ARG, "tile chunk");
    for (const OzRun &r : runs)
        BSG_REQUIRE(r.sh.nd >= 2 && r.sh.nd <= kOzMaxDigits && r.sh.nd * r.sh.np + 8 <= 512, BSG_ERR_UNSUPPORTED,
                    "Ozaki form: 2..8 digits, digits x padded block columns < 512");
    int *err = ctx->gemm_err_flag();
    auto launch = [&](unsigned long long *prof) {
        if (runs.size() > 1) {
            // every width up to 64 runs in the widest instantiation
            launch_oz<64, true>(ctx, runs, d_tiles, n_tiles, d_steps, alpha, err, prof, chunk, s);
            return;
        }
        switch (runs[0].sh.np) {
            case 8: launch_oz<8, false>(ctx, runs, d_tiles, n_tiles, d_steps, alpha, err, prof, chunk, s); break;
            case 16: launch_oz<16, false>(ctx, runs, d_tiles, n_tiles, d_steps, alpha, err, prof, chunk, s); break;
            case 24: launch_oz<24, false>(ctx, runs, d_tiles, n_tiles, d_steps, alpha, err, prof, chunk, s); break;
            case 32: launch_oz<32, false>(ctx, runs, d_tiles, n_tiles, d_steps, alpha, err, prof, chunk, s); break;
            case 40: launch_oz<40, false>(ctx, runs, d_tiles, n_tiles, d_steps, alpha, err, prof, chunk, s); break;
            case 48: launch_oz<48, false>(ctx, runs, d_tiles, n_tiles, d_steps, alpha, err, prof, chunk, s); break;
            case 56: launch_oz<56, false>(ctx, runs, d_tiles, n_tiles, d_steps, alpha, err, prof, chunk, s); break;
            case 64: launch_oz<64, false>(ctx, runs, d_tiles, n_tiles, d_steps, alpha, err, prof, chunk, s); break;
            default: throw Error{BSG_ERR_UNSUPPORTED, "Ozaki form supports block sizes up to 64"};
        }
    };
    if (!ctx->timing) {
        // no synchronization: the flag is read once at the end of the public call
        launch(nullptr);
        return;
    }
    DevBuf profbuf(8 * kOzProf, s);
    BSG_CUDA(cudaMemsetAsync(profbuf.p, 0, 8 * kOzProf, s));
    auto *prof = profbuf.as<unsigned long long>();
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    BSG_CUDA(cudaEventCreate(&e0));
    BSG_CUDA(cudaEventCreate(&e1));
    BSG_CUDA(cudaEventRecord(e0, s));
    launch(prof);
    BSG_CUDA(cudaEventRecord(e1, s));
    unsigned long long macs = 0, st[kOzProf] = {};
    if (d_macs) BSG_CUDA(cudaMemcpyAsync(&macs, d_macs, 8, cudaMemcpyDeviceToHost, s));
    BSG_CUDA(cudaMemcpyAsync(st, prof, sizeof(st), cudaMemcpyDeviceToHost, s));
    BSG_CUDA(cudaStreamSynchronize(s));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ctx->oz_ms += ms;
    ctx->oz_launches += 1;
    ctx->oz_useful_macs += (double)macs;
    for (int i = 0; i < kOzProf; ++i) ctx->oz_stall[i] += st[i];
    ctx->gemm_check();
}

void oz_run(bsg_ctx ctx, const OzShape &sh, const OzTile *d_tiles, size_t n_tiles, const OzStep *d_steps,
            const bf16 *a_img, const bf16 *b_img, double alpha, cudaStream_t s, const unsigned long long *d_macs,
            uint32_t chunk) {
    if (!n_tiles) return;
    oz_launch_timed(ctx, {OzRun{sh, a_img, b_img, n_tiles}}, d_tiles, n_tiles, d_steps, alpha, s, d_macs, chunk);
}

void oz_run_groups(bsg_ctx ctx, const std::vector<OzRun> &runs, const OzTile *d_tiles, size_t n_tiles,
                   const OzStep *d_steps, double alpha, cudaStream_t s, const unsigned long long *d_macs) {
    if (!n_tiles) return;
    std::vector<OzRun> live;  // runs with tiles (an empty run would only cost a table entry)
    for (const OzRun &r : runs)
        if (r.tile_end > (live.empty() ? 0 : live.back().tile_end)) live.push_back(r);
    oz_launch_timed(ctx, live, d_tiles, n_tiles, d_steps, alpha, s, d_macs, 1);
}

// ---------------------------------------------------------------------------
// operand splitting for BlockSparseMatrix operands
// ---------------------------------------------------------------------------

__device__ __forceinline__ int ext_of(size_t blk, size_t bs, size_t n) {
    return (int)(((blk + 1) * bs <= n) ? bs : n - blk * bs);
}

// digit image of op(A) block (ib, kb) stored at table index b (rows x k,
// padded to mp x kp)
__global__ void k_img_opA(double *const *__restrict__ tab, size_t a_nrb, int tA, ScreenGeom g,
                          const int *__restrict__ rexp, int mp, int kp, int nd, bf16 *__restrict__ img, size_t n) {
    const size_t b = oz_warp_id();
    if (b >= n) return;
    const double *blk = tab[b];
    if (!blk) return;
    const size_t sr = b % a_nrb, sc = b / a_nrb;
    const size_t ib = tA ? sc : sr, kb = tA ? sr : sc;
    const int rows = ext_of(ib, g.ibs, g.ni), k = ext_of(kb, g.kbs, g.nk);
    // op(A)(r, l): stored block column-major (rows x k, or k x rows when transposed)
    oz_block_image(blk, tA ? k : rows, tA != 0, rows, k, rexp + ib * g.ibs, mp, kp, nd,
                   img + b * nd * (size_t)mp * kp, true);
}

// digit image of op(B) block (kb, jb) stored at table index b, as np rows
// (output columns) x kp
__global__ void k_img_opB(double *const *__restrict__ tab, size_t b_nrb, int tB, ScreenGeom g,
                          const int *__restrict__ cexp, int np, int kp, int nd, bf16 *__restrict__ img, size_t n) {
    const size_t b = oz_warp_id();
    if (b >= n) return;
    const double *blk = tab[b];
    if (!blk) return;
    const size_t sr = b % b_nrb, sc = b / b_nrb;
    const size_t kb = tB ? sc : sr, jb = tB ? sr : sc;
    const int cols = ext_of(jb, g.jbs, g.nj), k = ext_of(kb, g.kbs, g.nk);
    // image row n, k l = op(B)(l, n): stored (k x cols) -> src[l + n*k]; transposed (cols x k) -> src[n + l*cols]
    oz_block_image(blk, tB ? cols : k, tB == 0, cols, k, cexp + jb * g.jbs, np, kp, nd,
                   img + b * nd * (size_t)np * kp, false);
}

// steps of every tile: k blocks where the B block exists and at least one
// slot's (A, B) pair survives the screen (the FP64 form's predicate)
__global__ void k_oz_steps(OzTile *__restrict__ tiles, size_t n_tiles, const uint32_t *__restrict__ tile_ib,
                           const uint32_t *__restrict__ tile_jb, double *const *__restrict__ A,
                           const double *__restrict__ An, size_t a_nrb, double *const *__restrict__ B,
                           const double *__restrict__ Bn, size_t b_nrb, ScreenGeom g, int R, OzStep *__restrict__ steps,
                           unsigned long long *__restrict__ macs, uint32_t a_base, uint32_t b_base) {
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_tiles) return;
    const uint32_t jb = tile_jb[t];
    uint32_t n = 0;
    unsigned long long m = 0;
    const unsigned long long cols = ext_of(jb, g.jbs, g.nj);
    OzStep *out = steps + tiles[t].s0;
    for (size_t kb = 0; kb < g.nkb; ++kb) {
        const size_t bi = g.tB ? jb + kb * b_nrb : kb + jb * b_nrb;
        if (!B[bi]) continue;
        OzStep st;
        st.bmask = kOzAllSub;
        st.b = b_base + (uint32_t)bi;
        bool any = false;
        for (int s = 0; s < kOzMaxSlots; ++s) {
            st.a[s] = kOzNone;
            if (s >= R) continue;
            const uint32_t ib = tile_ib[t * kOzMaxSlots + s];
            if (ib == kOzNone) continue;
            const size_t ai = g.tA ? kb + ib * a_nrb : ib + kb * a_nrb;
            if (!A[ai]) continue;
            if (!(__dmul_rn(An[ai], Bn[bi]) >= g.tpb)) continue;
            st.a[s] = a_base + (uint32_t)ai;
            m += (unsigned long long)ext_of(ib, g.ibs, g.ni) * cols * ext_of(kb, g.kbs, g.nk);
            any = true;
        }
        if (any) out[n++] = st;
    }
    tiles[t].ns = n;
    if (m) atomicAdd(macs, m);
}

// Row maxima of |op(A)| as bit patterns (non-negative doubles order like
// their bits), one warp per stored block, atomicMax into rowbits[row]
__global__ void k_rowmax_opA(double *const *__restrict__ tab, size_t nblk, size_t a_nrb, int tA, ScreenGeom g,
                             unsigned long long *__restrict__ rowbits) {
    const size_t b = oz_warp_id();
    if (b >= nblk) return;
    const double *blk = tab[b];
    if (!blk) return;
    const size_t sr = b % a_nrb, sc = b / a_nrb;
    const size_t ib = tA ? sc : sr, kb = tA ? sr : sc;
    const int rows = ext_of(ib, g.ibs, g.ni), k = ext_of(kb, g.kbs, g.nk);
    const int ld = tA ? k : rows;
    for (int r = threadIdx.x & 31; r < rows; r += 32) {
        long long mx = 0;
        for (int l = 0; l < k; ++l) {
            const long long v = oz_absbits(tA ? blk[l + (size_t)r * ld] : blk[r + (size_t)l * ld]);
            mx = v > mx ? v : mx;
        }
        if (mx) atomicMax(&rowbits[ib * g.ibs + r], (unsigned long long)mx);
    }
}

// column maxima of |op(B)|, one warp per stored block
__global__ void k_colmax_opB(double *const *__restrict__ tab, size_t nblk, size_t b_nrb, int tB, ScreenGeom g,
                             unsigned long long *__restrict__ colbits) {
    const size_t b = oz_warp_id();
    if (b >= nblk) return;
    const double *blk = tab[b];
    if (!blk) return;
    const size_t sr = b % b_nrb, sc = b / b_nrb;
    const size_t kb = tB ? sc : sr, jb = tB ? sr : sc;
    const int cols = ext_of(jb, g.jbs, g.nj), k = ext_of(kb, g.kbs, g.nk);
    const int ld = tB ? cols : k;
    for (int c = threadIdx.x & 31; c < cols; c += 32) {
        long long mx = 0;
        for (int l = 0; l < k; ++l) {
            const long long v = oz_absbits(tB ? blk[c + (size_t)l * ld] : blk[l + (size_t)c * ld]);
            mx = v > mx ? v : mx;
        }
        if (mx) atomicMax(&colbits[jb * g.jbs + c], (unsigned long long)mx);
    }
}

__global__ void k_bits_to_exp(const unsigned long long *__restrict__ bits, size_t n, int *__restrict__ exps) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) exps[i] = oz_exp_of_bits((long long)bits[i]);
}

void oz_operand_images(bsg_ctx ctx, bsg_bsm A, bsg_bsm B, const ScreenGeom &g, const OzShape &sh, int *rexp,
                       int *cexp, bf16 *aimg, bf16 *bimg) {
    cudaStream_t s = ctx->stream;
    const size_t nr = g.nib * g.ibs, nc = g.njb * g.jbs;
    DevBuf bits((nr + nc) * 8, s);
    auto *rb = bits.as<unsigned long long>(), *cb = rb + nr;
    BSG_CUDA(cudaMemsetAsync(bits.p, 0, (nr + nc) * 8, s));
    k_rowmax_opA<<<oz_img_grid(A->nblocks()), 32 * kOzImgWarps, 0, s>>>(A->dptr, A->nblocks(), A->nrb, g.tA, g, rb);
    k_colmax_opB<<<oz_img_grid(B->nblocks()), 32 * kOzImgWarps, 0, s>>>(B->dptr, B->nblocks(), B->nrb, g.tB, g, cb);
    if (nr) k_bits_to_exp<<<(unsigned)ceil_div(nr, (size_t)256), 256, 0, s>>>(rb, nr, rexp);
    if (nc) k_bits_to_exp<<<(unsigned)ceil_div(nc, (size_t)256), 256, 0, s>>>(cb, nc, cexp);
    ctx->note_launch(2);
    k_img_opA<<<oz_img_grid(A->nblocks()), 32 * kOzImgWarps, 0, s>>>(A->dptr, A->nrb, g.tA, g, rexp, sh.mp, sh.kp,
                                                                     sh.nd, aimg, A->nblocks());
    k_img_opB<<<oz_img_grid(B->nblocks()), 32 * kOzImgWarps, 0, s>>>(B->dptr, B->nrb, g.tB, g, cexp, sh.np, sh.kp,
                                                                     sh.nd, bimg, B->nblocks());
    ctx->note_launch(4);
    ctx->check_launch("ozaki split");
}

void oz_build_tiles(bsg_ctx ctx, const ScreenItems &si, const OzShape &sh, const int *rexp, const int *cexp,
                    uint32_t step_base, bool all_fresh, double *scratch, OzTilePlan &out) {
    const ScreenGeom &g = si.g;
    const auto &items = si.items;
    std::vector<OzTile> tiles;
    std::vector<uint32_t> tib, tjb;
    size_t i = 0;
    size_t slot_no = 0;
    const size_t blk_elems = g.ibs * g.jbs;
    while (i < items.size()) {
        OzTile T{};
        const uint32_t jb = si.item_jb[i];
        T.cexp = cexp + jb * g.jbs;
        T.cols = items[i].cols;
        const size_t base = tib.size();
        tib.resize(base + kOzMaxSlots, kOzNone);
        int sl = 0;
        while (i < items.size() && si.item_jb[i] == jb && sl < sh.R) {
            // scratch (autotuning trials): every slot writes its own scratch block
            T.c[sl] = scratch ? scratch + (slot_no++) * blk_elems : items[i].c;
            T.cnorm[sl] = scratch ? nullptr : items[i].c_norm;
            T.rows[sl] = items[i].rows;
            T.ldc[sl] = items[i].rows;
            T.rexp[sl] = rexp + si.item_ib[i] * g.ibs;
            if (items[i].fresh || all_fresh || scratch) T.fresh_mask |= 1u << sl;
            tib[base + sl] = si.item_ib[i];
            ++sl;
            ++i;
        }
        T.ns = 0;
        tiles.push_back(T);
        tjb.push_back(jb);
    }
    // super-tile order (Gr row groups x Gc block columns) keeps the digit
    // images of concurrently running tiles in L2
    const size_t Gr = 8, Gc = std::max<size_t>(1, 2 * (size_t)ctx->sm_count / Gr);
    std::vector<size_t> idx(tiles.size());
    for (size_t t = 0; t < idx.size(); ++t) idx[t] = t;
    auto key = [&](size_t t) {
        const size_t rg = tib[t * kOzMaxSlots] / (size_t)sh.R, jb = tjb[t];
        return std::make_tuple(rg / Gr, jb / Gc, rg % Gr, jb % Gc, rg, t);
    };
    std::sort(idx.begin(), idx.end(), [&](size_t a, size_t b) { return key(a) < key(b); });
    const size_t t0 = out.tiles.size();
    out.tiles.resize(t0 + tiles.size());
    out.tib.resize((t0 + tiles.size()) * kOzMaxSlots);
    out.tjb.resize(t0 + tiles.size());
    for (size_t n = 0; n < idx.size(); ++n) {
        out.tiles[t0 + n] = tiles[idx[n]];
        out.tiles[t0 + n].s0 = step_base + (uint32_t)(n * g.nkb);
        std::copy(tib.begin() + idx[n] * kOzMaxSlots, tib.begin() + (idx[n] + 1) * kOzMaxSlots,
                  out.tib.begin() + (t0 + n) * kOzMaxSlots);
        out.tjb[t0 + n] = tjb[idx[n]];
    }
}

void oz_launch_steps(bsg_ctx ctx, OzTile *d_tiles, size_t n_tiles, const uint32_t *d_tib, const uint32_t *d_tjb,
                     bsg_bsm A, bsg_bsm B, const ScreenGeom &g, int R, OzStep *d_steps, unsigned long long *d_macs,
                     uint32_t a_base, uint32_t b_base) {
    if (!n_tiles) return;
    k_oz_steps<<<(unsigned)ceil_div(n_tiles, 128), 128, 0, ctx->stream>>>(d_tiles, n_tiles, d_tib, d_tjb, A->dptr,
                                                                          A->dnorm, A->nrb, B->dptr, B->dnorm, B->nrb,
                                                                          g, R, d_steps, d_macs, a_base, b_base);
    ctx->note_launch();
    ctx->check_launch("ozaki steps");
}

void ozaki_screened(bsg_ctx ctx, bsg_bsm C, bsg_bsm A, bsg_bsm B, const ScreenGeom &g, const std::vector<GemmItem> &items,
                    const std::vector<uint32_t> &item_ib, const std::vector<uint32_t> &item_jb, double alpha,
                    int n_digits, cudaStream_t s) {
    if (items.empty()) return;
    (void)C;
    BSG_REQUIRE(g.ibs <= 64 && g.jbs <= 64 && g.kbs <= 64, BSG_ERR_UNSUPPORTED, "Ozaki form supports blocks up to 64");
    const int nd = oz_default_digits(n_digits, (int)g.ibs, (int)g.kbs, (int)g.jbs);
    const OzShape sh = oz_shape((int)g.ibs, (int)g.kbs, (int)g.jbs, nd);
    DevBuf rexp(g.nib * g.ibs * 4, s), cexp(g.njb * g.jbs * 4, s);
    DevBuf aimg(A->nblocks() * nd * (size_t)sh.mp * sh.kp * 2, s), bimg(B->nblocks() * nd * (size_t)sh.np * sh.kp * 2, s);
    oz_operand_images(ctx, A, B, g, sh, rexp.as<int>(), cexp.as<int>(), aimg.as<bf16>(), bimg.as<bf16>());
    ScreenItems si;
    si.g = g;
    si.items = items;
    si.item_ib = item_ib;
    si.item_jb = item_jb;
    OzTilePlan tp;
    oz_build_tiles(ctx, si, sh, rexp.as<int>(), cexp.as<int>(), 0, false, nullptr, tp);
    const size_t n_tiles = tp.tiles.size();
    BSG_REQUIRE(n_tiles * g.nkb < 0xffffffffull, BSG_ERR_UNSUPPORTED, "too many Ozaki steps in one call");
    DevBuf dt(n_tiles * sizeof(OzTile), s), dib(tp.tib.size() * 4, s), djb(tp.tjb.size() * 4, s),
        dst(n_tiles * g.nkb * sizeof(OzStep), s), dmacs(8, s);
    BSG_CUDA(cudaMemsetAsync(dmacs.p, 0, 8, s));
    BSG_CUDA(cudaMemcpyAsync(dt.p, tp.tiles.data(), n_tiles * sizeof(OzTile), cudaMemcpyHostToDevice, s));
    BSG_CUDA(cudaMemcpyAsync(dib.p, tp.tib.data(), tp.tib.size() * 4, cudaMemcpyHostToDevice, s));
    BSG_CUDA(cudaMemcpyAsync(djb.p, tp.tjb.data(), tp.tjb.size() * 4, cudaMemcpyHostToDevice, s));
    oz_launch_steps(ctx, dt.as<OzTile>(), n_tiles, dib.as<uint32_t>(), djb.as<uint32_t>(), A, B, g, sh.R,
                    dst.as<OzStep>(), dmacs.as<unsigned long long>(), 0, 0);
    oz_run(ctx, sh, dt.as<OzTile>(), n_tiles, dst.as<OzStep>(), aimg.as<bf16>(), bimg.as<bf16>(), alpha, s,
           dmacs.as<unsigned long long>());
    ctx->gemm_check();
}

// ---------------------------------------------------------------------------
// dense grid products X += P Q (the Strassen-Winograd leaves,
// strassen.hpp:311-323): n x n grids of bs x bs blocks, all blocks present
// ---------------------------------------------------------------------------

// exponent of every row of P (over the whole k range of its product); grid (product, rb)
__global__ void k_grid_rexp(double *const *__restrict__ P, size_t n, int bs, int *__restrict__ rexp) {
    const size_t i = blockIdx.x / n, rb = blockIdx.x % n;
    const int r = threadIdx.x;
    if (r >= bs) return;
    long long mx = 0;
    for (size_t kb = 0; kb < n; ++kb) {
        const double *blk = P[i * n * n + rb + kb * n];
        for (int l = 0; l < bs; ++l) {
            const long long b = oz_absbits(blk[r + (size_t)l * bs]);
            mx = b > mx ? b : mx;
        }
    }
    rexp[(i * n + rb) * bs + r] = oz_exp_of_bits(mx);
}

// exponent of every column of Q; grid (product, cb)
__global__ void k_grid_cexp(double *const *__restrict__ Q, size_t n, int bs, int *__restrict__ cexp) {
    const size_t i = blockIdx.x / n, cb = blockIdx.x % n;
    const int c = threadIdx.x;
    if (c >= bs) return;
    long long mx = 0;
    for (size_t kb = 0; kb < n; ++kb) {
        const double *blk = Q[i * n * n + kb + cb * n];
        for (int l = 0; l < bs; ++l) {
            const long long b = oz_absbits(blk[l + (size_t)c * bs]);
            mx = b > mx ? b : mx;
        }
    }
    cexp[(i * n + cb) * bs + c] = oz_exp_of_bits(mx);
}

// M-side images of P blocks, index i*n*n + rb + kb*n (a tile's slots are consecutive)
__global__ void k_grid_img_P(double *const *__restrict__ P, size_t n_blk, size_t n, int bs, const int *__restrict__ rexp,
                             OzShape sh, bf16 *__restrict__ img) {
    const size_t x = oz_warp_id();
    if (x >= n_blk) return;
    const size_t i = x / (n * n), rb = x % n;
    oz_block_image(P[x], bs, false, bs, bs, rexp + (i * n + rb) * bs, sh.mp, sh.kp, sh.nd,
                   img + x * (size_t)sh.nd * sh.mp * sh.kp, true);
}

// N-side images of Q blocks (image row = output column), index i*n*n + kb + cb*n
__global__ void k_grid_img_Q(double *const *__restrict__ Q, size_t n_blk, size_t n, int bs, const int *__restrict__ cexp,
                             OzShape sh, bf16 *__restrict__ img) {
    const size_t x = oz_warp_id();
    if (x >= n_blk) return;
    const size_t i = x / (n * n), cb = (x % (n * n)) / n;
    oz_block_image(Q[x], bs, true, bs, bs, cexp + (i * n + cb) * bs, sh.np, sh.kp, sh.nd,
                   img + x * (size_t)sh.nd * sh.np * sh.kp, false);
}

void ozaki_grid_products(bsg_ctx ctx, size_t n_prod, size_t n, const std::vector<double *> &X,
                         const std::vector<double *> &P, const std::vector<double *> &Q, int bs, int n_digits,
                         cudaStream_t s) {
    if (!n_prod || !n) return;
    BSG_REQUIRE(bs <= 64, BSG_ERR_UNSUPPORTED, "Ozaki form supports blocks up to 64");
    const size_t nn = n * n, n_blk = n_prod * nn;
    BSG_REQUIRE(X.size() == n_blk && P.size() == n_blk && Q.size() == n_blk, BSG_ERR_ARG, "grid tables");
    const int nd = oz_default_digits(n_digits, bs, bs, bs);
    const OzShape sh = oz_shape(bs, bs, bs, nd);
    DevBuf dP(n_blk * 8, s), dQ(n_blk * 8, s), rexp(n_prod * n * bs * 4, s), cexp(n_prod * n * bs * 4, s);
    DevBuf aimg(n_blk * nd * (size_t)sh.mp * sh.kp * 2, s), bimg(n_blk * nd * (size_t)sh.np * sh.kp * 2, s);
    BSG_CUDA(cudaMemcpyAsync(dP.p, P.data(), n_blk * 8, cudaMemcpyHostToDevice, s));
    BSG_CUDA(cudaMemcpyAsync(dQ.p, Q.data(), n_blk * 8, cudaMemcpyHostToDevice, s));
    const unsigned tb = (unsigned)std::max(32, round_up(bs, 32));
    k_grid_rexp<<<(unsigned)(n_prod * n), tb, 0, s>>>(dP.as<double *>(), n, bs, rexp.as<int>());
    k_grid_cexp<<<(unsigned)(n_prod * n), tb, 0, s>>>(dQ.as<double *>(), n, bs, cexp.as<int>());
    k_grid_img_P<<<oz_img_grid(n_blk), 32 * kOzImgWarps, 0, s>>>(dP.as<double *>(), n_blk, n, bs, rexp.as<int>(), sh,
                                                                 aimg.as<bf16>());
    k_grid_img_Q<<<oz_img_grid(n_blk), 32 * kOzImgWarps, 0, s>>>(dQ.as<double *>(), n_blk, n, bs, cexp.as<int>(), sh,
                                                                 bimg.as<bf16>());
    ctx->note_launch(4);
    ctx->check_launch("ozaki grid split");
    // tiles (product, block column cb, R consecutive block rows), steps over kb
    const size_t ng = ceil_div(n, (size_t)sh.R);
    std::vector<OzTile> tiles;
    std::vector<OzStep> steps;
    tiles.reserve(n_prod * n * ng);
    steps.reserve(n_prod * n * ng * n);
    for (size_t i = 0; i < n_prod; ++i)
        for (size_t cb = 0; cb < n; ++cb)
            for (size_t g = 0; g < ng; ++g) {
                OzTile T{};
                for (int sl = 0; sl < sh.R; ++sl) {
                    const size_t rb = g * sh.R + sl;
                    if (rb >= n) break;
                    T.c[sl] = X[i * nn + rb + cb * n];
                    T.rows[sl] = bs;
                    T.ldc[sl] = bs;
                    T.rexp[sl] = rexp.as<int>() + (i * n + rb) * bs;
                }
                T.cols = bs;
                T.cexp = cexp.as<int>() + (i * n + cb) * bs;
                T.fresh_mask = 0;  // X += P Q
                T.s0 = (uint32_t)steps.size();
                T.ns = (uint32_t)n;
                for (size_t kb = 0; kb < n; ++kb) {
                    OzStep st;
        st.bmask = kOzAllSub;
                    st.b = (uint32_t)(i * nn + kb + cb * n);
                    for (int sl = 0; sl < kOzMaxSlots; ++sl) {
                        const size_t rb = g * sh.R + sl;
                        st.a[sl] = (sl < sh.R && rb < n) ? (uint32_t)(i * nn + rb + kb * n) : kOzNone;
                    }
                    steps.push_back(st);
                }
                tiles.push_back(T);
            }
    BSG_REQUIRE(steps.size() < 0xffffffffull && n_blk < 0xffffffffull, BSG_ERR_UNSUPPORTED, "grid products too large");
    DevBuf dt(tiles.size() * sizeof(OzTile), s), dst(steps.size() * sizeof(OzStep), s), dmacs(8, s);
    BSG_CUDA(cudaMemcpyAsync(dt.p, tiles.data(), tiles.size() * sizeof(OzTile), cudaMemcpyHostToDevice, s));
    BSG_CUDA(cudaMemcpyAsync(dst.p, steps.data(), steps.size() * sizeof(OzStep), cudaMemcpyHostToDevice, s));
    const unsigned long long macs = (unsigned long long)n_prod * n * n * n * bs * bs * bs;
    BSG_CUDA(cudaMemcpyAsync(dmacs.p, &macs, 8, cudaMemcpyHostToDevice, s));
    oz_run(ctx, sh, dt.as<OzTile>(), tiles.size(), dst.as<OzStep>(), aimg.as<bf16>(), bimg.as<bf16>(), 1.0, s,
           dmacs.as<unsigned long long>());
    ctx->gemm_check();  // also keeps the host tables alive until the copies are done
}

}  // namespace bsg
