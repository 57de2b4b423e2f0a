// Host side of the GB300 engine: device buffers, the per-substep launch
// sequence, CUDA-graph replay, and the C ABI declared in include/suna.h.
//
// A World holds one or more independent 2D scenes in one set of device
// buffers (see world.cuh). The single-scene engine (sn_engine, the drop-in for
// the reference's Engine, src/engine.js:3523) is a World with one scene; the
// batched engine (sn_batch) is the same World with many.
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstddef>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/suna.h"
#include "ckptpool.h"
#include "radix.cuh"
#include "sim2d.cuh"
#include "rigid.cuh"
#include <cmath>

using namespace sn;
using namespace sn::d2;

namespace {

constexpr int32_t VMAX = 65536;
constexpr int32_t MAX_POS = 134217728;
constexpr int32_t KERNEL_H = 163840;
constexpr uint32_t FLAG_MASK = 7u;
constexpr uint32_t SPAWN_FLAG_MASK = 1u | 4u;

// A queued disc impulse (applyImpulse, src/engine.js:6077-6098).
struct ImpulseEv {
  uint32_t at;       // scene substep index before which it applies
  int32_t cx, cy, r, ix, iy;
  uint32_t limit;
  uint32_t pad;
};

struct EvPar {
  uint32_t begin, end, cursor, pad;
};

// Device impulse: one CTA per scene; due events apply in queue order, hits
// counted in slot order with a block-wide scan, first `limit` hits only.
// The disc test is the reference's JS arithmetic: IEEE doubles, each product
// and the sum rounded to nearest, no fused multiply-add, then !(s > r*r).
__device__ __forceinline__ bool in_disc_f64(int32_t px, int32_t py, const ImpulseEv& ev) {
  double dx = (double)px - (double)ev.cx;
  double dy = (double)py - (double)ev.cy;
  double r = (double)ev.r;
  double s = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
  return !(s > __dmul_rn(r, r));
}
// The same decision, taken in exact 64-bit integers wherever the doubles'
// rounding cannot change it (a filtered exact predicate). With X = dx^2 + dy^2
// and R = r^2 exact, each rounding to nearest moves a value by at most 2^-53
// of itself, so s lies within X * 3 * 2^-53 of X and r*r within R * 2^-53 of
// R; a gap |X - R| above (X >> 50) + (R >> 50) + 2 exceeds both, and the
// exact comparison gives the doubles' answer. Near-ties (and |dx| or |dy| at
// or above 2^31, where X could leave u64) take the double path.
__device__ __forceinline__ bool in_disc(int32_t px, int32_t py, const ImpulseEv& ev) {
  const int64_t dx = (int64_t)px - ev.cx, dy = (int64_t)py - ev.cy;
  const uint64_t ax = (uint64_t)(dx < 0 ? -dx : dx), ay = (uint64_t)(dy < 0 ? -dy : dy);
  if ((ax | ay) >> 31) return in_disc_f64(px, py, ev);
  const uint64_t X = ax * ax + ay * ay;
  const uint64_t R = (uint64_t)((int64_t)ev.r * ev.r);
  const uint64_t m = (X >> 50) + (R >> 50) + 2u;
  if (X > R + m) return false;
  if (X + m < R) return true;
  return in_disc_f64(px, py, ev);
}

// Exclusive block-wide prefix sum of v (every thread of the CTA calls it);
// *total receives the block's sum.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* total) {
  __shared__ uint32_t wsum[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (int)(blockDim.x >> 5);
  uint32_t inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) wsum[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < nw ? wsum[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += t;
    }
    wsum[lane] = w;  // inclusive over warps
  }
  __syncthreads();
  const uint32_t before = warp ? wsum[warp - 1] : 0u;
  *total = wsum[nw - 1];
  __syncthreads();  // wsum is reused by the next call
  return before + inc - v;
}

// One disc impulse over scene S's fluid particles (every thread of the CTA
// calls it). The hits are ranked in slot order: each thread owns a
// contiguous slot range, tests it (positions read eight at a time, the hits
// kept as a bit mask when the range is at most 64 slots), and a block scan
// gives each thread the rank of its first hit; the first `limit` hits get the
// impulse. Returns min(hits, limit).
__device__ uint32_t apply_event(Bufs b, const ScenePar& S, const ImpulseEv& ev) {
  const uint32_t n = S.nFluid, T = blockDim.x;
  const uint32_t per = (n + T - 1) / T;
  const uint32_t lo = min(n, threadIdx.x * per), hi = min(n, lo + per);
  int32_t* base = b.state + (size_t)S.slotBase * 8;
  auto pos = [&](uint32_t i) { return *reinterpret_cast<const int2*>(base + (size_t)i * 8); };
  uint32_t cnt = 0;
  uint64_t mask = 0;
  const bool masked = per <= 64u;
  uint32_t i = lo;
  for (; i + 8 <= hi; i += 8) {
    int2 q[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) q[j] = pos(i + j);
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const bool h = in_disc(q[j].x, q[j].y, ev);
      cnt += h ? 1u : 0u;
      if (masked && h) mask |= 1ull << (i + j - lo);
    }
  }
  for (; i < hi; ++i) {
    const int2 q = pos(i);
    const bool h = in_disc(q.x, q.y, ev);
    cnt += h ? 1u : 0u;
    if (masked && h) mask |= 1ull << (i - lo);
  }
  uint32_t total = 0;
  uint32_t rank = block_exclusive_scan(cnt, &total);
  auto kick = [&](uint32_t k) {
    int32_t* w = base + (size_t)k * 8;
    int64_t vx = (int64_t)w[2] + ev.ix, vy = (int64_t)w[3] + ev.iy;
    vx = vx < -VMAX ? -VMAX : (vx > VMAX ? VMAX : vx);
    vy = vy < -VMAX ? -VMAX : (vy > VMAX ? VMAX : vy);
    w[2] = (int32_t)vx;
    w[3] = (int32_t)vy;
  };
  if (cnt && rank < ev.limit) {
    if (masked) {
      for (; mask && rank < ev.limit; mask &= mask - 1u, ++rank) kick(lo + (uint32_t)(__ffsll((long long)mask) - 1));
    } else {
      for (uint32_t k = lo; k < hi && rank < ev.limit; ++k) {
        const int2 q = pos(k);
        if (!in_disc(q.x, q.y, ev)) continue;
        kick(k);
        ++rank;
      }
    }
  }
  __syncthreads();  // the next event of the scene reads these velocities
  return min(total, ev.limit);
}

// One CTA of IMPULSE_THREADS per scene: the disc test covers the scene's
// particles IMPULSE_THREADS at a time, in slot order (the hit ranks).
constexpr int IMPULSE_THREADS = 1024;
__global__ void __launch_bounds__(IMPULSE_THREADS) k_impulse_sched(Bufs b, const ImpulseEv* __restrict__ evs,
                                                       EvPar* __restrict__ ep) {
  uint32_t s = blockIdx.x;
  if (s >= b.world->numScenes) return;
  const ScenePar& S = b.scenes[s];
  if (!S.active) return;
  uint32_t cur = ep[s].cursor;
  const uint32_t end = ep[s].end;
  const uint32_t now = S.substep;
  while (cur < end && evs[cur].at <= now) {
    ImpulseEv ev = evs[cur];
    if (ev.at == now) apply_event(b, S, ev);
    ++cur;
    __syncthreads();
  }
  __syncthreads();
  if (threadIdx.x == 0) ep[s].cursor = cur;
}

__global__ void __launch_bounds__(256) k_impulse_now(Bufs b, uint32_t s, ImpulseEv ev, uint32_t* hitsOut) {
  const ScenePar& S = b.scenes[s];
  uint32_t h = apply_event(b, S, ev);
  if (threadIdx.x == 0) *hitsOut = h;
}

// The last substep's density (solveA's rho, the reference's Derived.rho,
// src/sim.wgsl:200) and neighbour count (nbrN's count field) of each slot of
// one scene, in slot order; wall slots read 0. Valid while the sorted-space
// arrays still belong to the slots (no edit since the substep).
__global__ void __launch_bounds__(256) k_slot_fields(Bufs b, uint32_t slotBase, uint32_t n, uint32_t nFluid,
                                                     int32_t* __restrict__ rho, uint32_t* __restrict__ nbr) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t p = b.inv[slotBase + i];
    const bool fluid = i < nFluid;
    rho[i] = fluid ? b.RX[p].x : 0;
    nbr[i] = fluid ? (b.NBRN[p] & NBRN_COUNT) : 0u;
  }
}

// eraseWhere (src/engine.js:6460-6650) on the device, for a scene without
// bodies. k_erase_rank: one CTA; each thread takes a contiguous range of the
// keep flags, and a block scan gives every survivor its new index in slot
// order (oldToNew[i], -1 for an erased particle; *kept = the survivors).
__global__ void __launch_bounds__(1024) k_erase_rank(const uint8_t* __restrict__ keep, uint32_t n,
                                                     int32_t* __restrict__ oldToNew, uint32_t* __restrict__ kept) {
  const uint32_t T = blockDim.x, per = (n + T - 1) / T;
  const uint32_t lo = min(n, threadIdx.x * per), hi = min(n, lo + per);
  uint32_t cnt = 0;
  for (uint32_t i = lo; i < hi; ++i) cnt += keep[i] ? 1u : 0u;
  uint32_t total = 0;
  uint32_t r = block_exclusive_scan(cnt, &total);
  for (uint32_t i = lo; i < hi; ++i) oldToNew[i] = keep[i] ? (int32_t)r++ : -1;
  if (threadIdx.x == 0) *kept = total;
}
// The survivors' state words and stAcc, then the boundary block after them,
// written at their new slots into scratch; newToOld[k] = survivor k's old slot.
__global__ void __launch_bounds__(256) k_erase_move(const int32_t* __restrict__ state, const int2* __restrict__ stacc,
                                                    const int32_t* __restrict__ oldToNew, uint32_t n, uint32_t oldF,
                                                    uint32_t newF, int4* __restrict__ outState,
                                                    int2* __restrict__ outStacc, uint32_t* __restrict__ newToOld) {
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    const int32_t d = j < oldF ? oldToNew[j] : (int32_t)(newF + (j - oldF));
    if (d < 0) continue;
    const int4* src = reinterpret_cast<const int4*>(state + (size_t)j * 8);
    outState[2 * (size_t)d] = src[0];
    outState[2 * (size_t)d + 1] = src[1];
    outStacc[d] = stacc[j];
    if (j < oldF) newToOld[d] = j;
  }
}
// Survivor k's bond row from its old row: tombstones and bonds to erased
// particles dropped, partners renumbered (a partner index past the old fluid
// count is dropped too); rows from the survivor count up to the old fluid
// count come out empty.
__global__ void __launch_bounds__(256) k_erase_bonds(const uint32_t* __restrict__ bond,
                                                     const int32_t* __restrict__ oldToNew,
                                                     const uint32_t* __restrict__ newToOld, uint32_t oldF,
                                                     uint32_t newF, uint32_t* __restrict__ out) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < oldF; k += gridDim.x * blockDim.x) {
    uint32_t* o = out + (size_t)k * BOND_CAP;
    uint32_t c = 0;
    if (k < newF) {
      const uint32_t* row = bond + (size_t)newToOld[k] * BOND_CAP;
      for (int q = 0; q < BOND_CAP; ++q) {
        const uint32_t w = row[q];
        if (w == 0u) break;
        if (w & BOND_TOMB) continue;
        const uint32_t j = w & BOND_J_MASK;
        const int32_t nj = j < oldF ? oldToNew[j] : -1;
        if (nj < 0) continue;
        o[c++] = (w & BOND_L0_MASK) | (uint32_t)nj;
      }
    }
    for (; c < (uint32_t)BOND_CAP; ++c) o[c] = 0u;
  }
}

// Per material row, the words loadScene derives (src/engine.js:3855-3880):
// the flag bits a fluid / wall particle of that row gets (FLAG_DEAD for a
// phantom row, FLAG_SEAL for a seal-class row, the scene weld tag for a fluid
// particle of a welding row) and the row's fuel0.
struct LoadTables {
  uint32_t fluidFl[MAT_MAX], wallFl[MAT_MAX];
  int32_t fuel0[MAT_MAX];
};
// The uploaded arrays (SoA, see upload_scene): pos 2n, vel 2n, mat n, flags n,
// temp n, fuel n; `present` bit 0/1/2: flags/temp/fuel given.
// loadScene's per-particle checks (the same tests, in the same order, as the
// host's validate_particle): res[0] = the first failing particle, res[1..2] =
// the mask of material rows present.
__global__ void __launch_bounds__(256) k_load_check(const int32_t* __restrict__ raw, uint32_t n, uint32_t nFluid,
                                                    uint32_t matCount, uint32_t present, LoadTables T,
                                                    uint32_t* __restrict__ res) {
  uint64_t seen = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t m = (uint32_t)raw[4 * (size_t)n + i];
    const int32_t px = raw[2 * (size_t)i], py = raw[2 * (size_t)i + 1];
    const int32_t lo = i < nFluid ? 0 : -MAX_POS;
    const uint32_t fl = (present & 1u) ? (uint32_t)raw[5 * (size_t)n + i] : 0u;
    bool bad = m >= matCount || px < lo || px > MAX_POS || py < lo || py > MAX_POS || (fl & ~FLAG_MASK);
    if (!bad && (present & 2u)) {
      const int32_t t = raw[6 * (size_t)n + i];
      bad = t < TEMP_MIN || t > TEMP_MAX;
    }
    if (!bad && (present & 4u)) bad = raw[7 * (size_t)n + i] < 0;
    if (!bad && (fl & FLAG_DEAD) && !(T.wallFl[m] & FLAG_DEAD)) bad = true;
    if (bad) atomicMin(res, i);
    else seen |= 1ull << m;
  }
  const uint32_t lo32 = __reduce_or_sync(0xffffffffu, (uint32_t)seen);
  const uint32_t hi32 = __reduce_or_sync(0xffffffffu, (uint32_t)(seen >> 32));
  if ((threadIdx.x & 31u) == 0u) {
    if (lo32) atomicOr(res + 1, lo32);
    if (hi32) atomicOr(res + 2, hi32);
  }
}
// loadScene's packing (src/engine.js:3855-3880) of the checked arrays into the
// scene's cap slots of state words; slots past n are zero.
__global__ void __launch_bounds__(256) k_load_pack(const int32_t* __restrict__ raw, uint32_t n, uint32_t nFluid,
                                                   uint32_t cap, uint32_t present, LoadTables T,
                                                   int32_t* __restrict__ state) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += gridDim.x * blockDim.x) {
    int4 a = make_int4(0, 0, 0, 0), c = make_int4(0, 0, 0, 0);
    if (i < n) {
      const uint32_t m = (uint32_t)raw[4 * (size_t)n + i];
      const uint32_t given = (present & 1u) ? (uint32_t)raw[5 * (size_t)n + i] : 0u;
      a = make_int4(raw[2 * (size_t)i], raw[2 * (size_t)i + 1], raw[2 * (size_t)n + 2 * (size_t)i],
                    raw[2 * (size_t)n + 2 * (size_t)i + 1]);
      c = make_int4((int32_t)m, (int32_t)(given | (i < nFluid ? T.fluidFl[m] : T.wallFl[m])),
                    (present & 2u) ? raw[6 * (size_t)n + i] : AMBIENT,
                    (present & 4u) ? raw[7 * (size_t)n + i] : T.fuel0[m]);
    }
    int4* w4 = reinterpret_cast<int4*>(state + (size_t)i * 8);
    w4[0] = a;
    w4[1] = c;
  }
}

__global__ void __launch_bounds__(256) k_fill_u32(uint32_t* __restrict__ out, uint32_t n, uint32_t v) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = v;
}

template <typename T>
T* dalloc(size_t count, std::string& err) {
  if (count == 0) count = 1;
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, count * sizeof(T));
  if (e != cudaSuccess) {
    err = std::string("cudaMalloc: ") + cudaGetErrorString(e);
    return nullptr;
  }
  // The zeroing runs on the legacy default stream, which does not order with
  // the engine's non-blocking stream: finish it before anything is queued there.
  cudaMemset(p, 0, count * sizeof(T));
  cudaDeviceSynchronize();
  return static_cast<T*>(p);
}

struct SceneHost {
  bool used = false, loaded = false;
  uint32_t slotBase = 0, cap = 0;
  uint32_t n = 0, nFluid = 0;
  uint32_t gridW = 1, gridH = 1, cellShift = 18, cellTotal = 1;
  int32_t domW = 0, domH = 0;
  uint64_t substeps = 0;
  // the loaded scene's boundary block: spawnFluid and setWalls re-pack it
  std::vector<int32_t> bpos, btemp, bfuel;
  std::vector<uint32_t> bmat;
  uint64_t matSeen = 0;  // the material rows any particle of the scene has worn (loaded or spawned)
  uint32_t nFluid0 = 0;
  uint32_t nInit = 0;  // particles of the last loadScene (their positions are in World::initPos)
  bool hasTemp = false, hasFuel = false;
  uint32_t weldSeq = 1;                   // _weldSeq: the loaded scene holds tag sequence 1
  uint32_t weldHold = 0, weldHoldSeq = 0;  // the gesture held open
  uint32_t fuseTag = 0, lastWeldTag = 0;
  bool wallsOn = true;
  std::vector<ImpulseEv> events;
  uint32_t consumed = 0;  // events already applied (at < substeps)
};

}  // namespace

struct World {
  int device = 0;
  cudaStream_t st = nullptr;
  // A side stream for work that runs beside the main chain: each colour
  // pass's copy of the other colours forks onto it and joins before the next
  // pass (inside the captured graph, a parallel branch).
  cudaStream_t st2 = nullptr;
  cudaEvent_t evFork = nullptr, evJoin = nullptr;
  bool debug = false, chainOn = true;
  uint32_t iters = 4;
  uint32_t capSlots = 0, maxCells = 0, maxScenes = 0;
  int numSMs = 152;
  std::string err;
  int32_t hmats[MAT_MAX * MAT_WORDS];  // the device image (grav scaled by gravQ)
  int32_t hauth[MAT_MAX * MAT_WORDS];  // the rows as authored or minted
  uint32_t matCount = 0, authoredCount = 0;
  int32_t gravQ = 65536;               // setGravityScale, Q16
  std::vector<SceneHost> sh;
  std::vector<ScenePar> hpar;
  WorldPar hw{};
  Bufs b{};
  uint32_t *tmpK = nullptr, *tmpV = nullptr, *hist = nullptr, *hits = nullptr;
  uint32_t* accTmp = nullptr;
  BoxChunk* boxChunks = nullptr;  // [capSlots / CELL_CHUNK + capSlots / CELL_BIG + 1] (k_cellbox)
  ImpulseEv* devEv = nullptr;
  size_t devEvCap = 0;
  EvPar* devEp = nullptr;
  bool eventsDirty = false, anyEvents = false;
  bool hasFriction = false, hasBonds = false, hasSeal = false;
  bool layoutDirty = true;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  bool graphValid = false;
  bool useGraph = true;
  int lanesOverride = 0;  // 0 = choose from the active particle count
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  float lastMs = 0.f;
  uint64_t lastLaunches = 0;
  uint64_t launchesPerSubstep = 0;

  bool fail(const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    err = buf;
    return false;
  }
  bool cuda_ok(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return true;
    return fail("%s: %s", what, cudaGetErrorString(e));
  }

  ~World() {
    if (gexec) cudaGraphExecDestroy(gexec);
    if (graph) cudaGraphDestroy(graph);
    void* ptrs[] = {b.state, b.stacc, b.predSlot, b.sceneOf, b.keys, b.inv, b.bond, b.bondCand, b.skey,
                    b.sslot, b.cellStart, b.PL, b.PL2, b.RX, b.NQ, b.POS, b.SCN, b.DP, b.HEAT, b.CORR, b.NBR,
                    b.NBRL, b.NBRN, (void*)b.tiles, b.TR, b.OVF, b.CB,
                    (void*)b.luts, (void*)b.WG, (void*)b.CA, (void*)b.mats, (void*)b.rcp,
                    b.scenes, b.world, b.acc, b.accLast, b.chain, b.dbg, b.err, b.work, tmpK, tmpV, hist,
                    hits, accTmp, devEv, devEp, boxChunks, upl, uplRes, barBuf, eraseBuf, initPos};
    for (void* p : ptrs)
      if (p) cudaFree(p);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (evFork) cudaEventDestroy(evFork);
    if (evJoin) cudaEventDestroy(evJoin);
    if (st2) cudaStreamDestroy(st2);
    if (st) cudaStreamDestroy(st);
  }

  bool init(const sn_opts* o, uint32_t scenesCap) {
    if (!o) return fail("opts is NULL");
    if (o->max_particles == 0) return fail("max_particles must be > 0");
    if (o->iters < 1 || o->iters > 16) return fail("iters = %u outside 1..16", o->iters);
    if (!o->luts || !o->mats) return fail("luts and mats are required");
    if (o->mat_count < 1 || o->mat_count > (uint32_t)MAT_MAX) return fail("mat_count must be 1..64");
    device = o->device;
    if (!cuda_ok(cudaSetDevice(device), "cudaSetDevice")) return false;
    cudaDeviceGetAttribute(&numSMs, cudaDevAttrMultiProcessorCount, device);
    debug = o->debug != 0;
    chainOn = o->chain != 0;
    if (o->lanes != 0 && o->lanes != 1 && o->lanes != 2 && o->lanes != 4 && o->lanes != 8)
      return fail("lanes must be 0, 1, 2, 4 or 8");
    lanesOverride = (int)o->lanes;
    autoLanes = o->lanes == 0;
    iters = o->iters;
    capSlots = o->max_particles;
    maxCells = o->max_cells ? o->max_cells : (1u << 20);
    maxScenes = scenesCap;
    std::memset(hmats, 0, sizeof(hmats));
    std::memcpy(hmats, o->mats, sizeof(int32_t) * MAT_WORDS * o->mat_count);
    std::memcpy(hauth, hmats, sizeof(hauth));
    matCount = authoredCount = o->mat_count;
    for (uint32_t m = 0; m < matCount; ++m) {
      const int32_t* r = hmats + m * MAT_WORDS;
      if (r[M_eps] < 32768) return fail("mats[%u].eps < 32768", m);
      if (r[M_dpMax] <= 0) return fail("mats[%u].dpMax <= 0", m);
      for (int f : {M_meltTo, M_freezeTo, M_boilTo, M_condTo, M_burnTo, M_splitTo, M_corrTo})
        if (r[f] < 0 || (uint32_t)r[f] >= matCount) return fail("mats[%u] names a product outside the table", m);
      // §29 words (src/engine.js:3247-3256): only seal-class rows carry them
      const bool sealRow = r[M_bondK] != 0 && r[M_bondReform] == 0 && r[M_solidMode] != 0 && r[M_phantom] == 0;
      if (r[M_burstP] < 0) return fail("mats[%u].burstP < 0", m);
      if (r[M_sealMode] != 0 && r[M_sealMode] != 1) return fail("mats[%u].sealMode must be 0 or 1", m);
      if (!sealRow && (r[M_burstP] != 0 || r[M_sealMode] != 0))
        return fail("mats[%u] is not seal-class but carries burstP/sealMode", m);
    }
    if (!cuda_ok(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "stream")) return false;
    if (!cuda_ok(cudaStreamCreateWithFlags(&st2, cudaStreamNonBlocking), "stream")) return false;
    cudaEventCreate(&ev0);
    cudaEventCreate(&ev1);
    cudaEventCreateWithFlags(&evFork, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&evJoin, cudaEventDisableTiming);
    size_t C = capSlots;
    b.state = dalloc<int32_t>(C * 8, err);
    b.stacc = dalloc<int2>(C, err);
    b.predSlot = dalloc<int2>(C, err);
    b.sceneOf = dalloc<uint32_t>(C, err);
    b.keys = dalloc<uint32_t>(C, err);
    b.inv = dalloc<uint32_t>(C, err);
    b.bond = dalloc<uint32_t>(C * BOND_CAP, err);
    b.bondCand = dalloc<uint32_t>(C * BOND_CAP, err);
    b.skey = dalloc<uint32_t>(C, err);
    b.sslot = dalloc<uint32_t>(C, err);
    b.PL = dalloc<int4>(C, err);
    b.PL2 = dalloc<int4>(C, err);
    b.RX = dalloc<int4>(C, err);
    b.NQ = dalloc<int4>(C, err);
    b.POS = dalloc<int2>(C, err);
    b.SCN = dalloc<uint32_t>(C, err);
    b.DP = dalloc<int2>(C, err);
    b.HEAT = dalloc<int32_t>(C, err);
    b.CORR = dalloc<int32_t>(C, err);
    b.NBR = dalloc<uint32_t>(C * MAXNBR, err);
    b.NBRL = dalloc<uint16_t>(C * MAXNBR, err);
    b.NBRN = dalloc<uint32_t>(C, err);
    b.nbrStride = (uint32_t)C;
    uint16_t* drcp = dalloc<uint16_t>(32768, err);
    int32_t* dl = dalloc<int32_t>(LUT_WORDS, err);
    int2* dwg = dalloc<int2>(TN, err);
    int2* dca = dalloc<int2>(TN, err);
    int32_t* dm = dalloc<int32_t>(MAT_MAX * MAT_WORDS, err);
    b.scenes = dalloc<ScenePar>(scenesCap, err);
    b.world = dalloc<WorldPar>(1, err);
    b.acc = dalloc<uint32_t>((size_t)scenesCap * 8, err);
    b.accLast = dalloc<uint32_t>((size_t)scenesCap * 8, err);
    b.chain = dalloc<uint32_t>((size_t)scenesCap * 8, err);
    b.dbg = dalloc<uint32_t>(16, err);
    b.err = dalloc<uint32_t>(4, err);
    b.work = dalloc<uint32_t>(8, err);
    barBuf = dalloc<uint32_t>(2, err);
    tmpK = dalloc<uint32_t>(C, err);
    tmpV = dalloc<uint32_t>(C, err);
    hist = dalloc<uint32_t>(radix::hist_words((uint32_t)C), err);
    hits = dalloc<uint32_t>(1, err);
    accTmp = dalloc<uint32_t>((size_t)scenesCap * 8, err);
    boxChunks = dalloc<BoxChunk>(C / CELL_CHUNK + C / CELL_BIG + 1, err);
    devEp = dalloc<EvPar>(scenesCap, err);
    b.rbody = dalloc<int32_t>((size_t)RG_MAX_BODIES * RG_BODY_WORDS, err);
    b.rdrv = dalloc<int32_t>((size_t)RG_MAX_BODIES * RG_DRIVER_WORDS, err);
    b.rest = dalloc<int2>(C, err);
    b.rmark = dalloc<uint32_t>(C, err);
    int32_t* dcos = dalloc<int32_t>(RG_COS_N, err);
    if (!err.empty()) return false;
    {
      int32_t T[RG_COS_N];
      build_cos_table(T);
      cudaMemcpy(dcos, T, sizeof(T), cudaMemcpyHostToDevice);
      b.cosT = dcos;
    }
    for (int i = 4 * TN; i < 5 * TN; ++i)
      if (o->luts[i] != 0) return fail("the s_corr kernel table must be all zero (scorrK = 0 in the frozen tables)");
    cudaMemcpy(dl, o->luts, sizeof(int32_t) * LUT_WORDS, cudaMemcpyHostToDevice);
    {
      std::vector<int2> wg(TN), ca(TN);
      for (int i = 0; i < TN; ++i) {
        wg[i] = make_int2(o->luts[i], o->luts[TN + i]);
        ca[i] = make_int2(o->luts[2 * TN + i], o->luts[3 * TN + i]);
      }
      cudaMemcpy(dwg, wg.data(), sizeof(int2) * TN, cudaMemcpyHostToDevice);
      cudaMemcpy(dca, ca.data(), sizeof(int2) * TN, cudaMemcpyHostToDevice);
    }
    b.WG = dwg;
    b.CA = dca;
    cudaMemcpy(dm, hmats, sizeof(hmats), cudaMemcpyHostToDevice);
    {
      std::vector<uint16_t> rc(32768);
      for (uint32_t dn = 32768; dn < 65536; ++dn) rc[dn - 32768] = (uint16_t)((1u << 30) / dn);
      cudaMemcpy(drcp, rc.data(), 65536, cudaMemcpyHostToDevice);
    }
    b.luts = dl;
    b.mats = dm;
    b.rcp = drcp;
    sh.assign(scenesCap, SceneHost{});
    hpar.assign(scenesCap, ScenePar{});
    return cuda_ok(cudaDeviceSynchronize(), "init");
  }

  const int32_t* row(uint32_t m) const { return hmats + m * MAT_WORDS; }
  bool seal_row(uint32_t m) const {
    const int32_t* r = row(m);
    return r[M_bondK] != 0 && r[M_bondReform] == 0 && r[M_solidMode] != 0 && r[M_phantom] == 0;
  }
  bool spawn_welds(uint32_t m) const { return row(m)[M_bondGroup] >= 0 && row(m)[M_bondReform] == 0; }
  // Which optional passes the loaded rows (and every row a transition can turn
  // them into) need.
  void update_features() {
    std::vector<bool> seen(matCount, false);
    std::vector<uint32_t> stack;
    for (auto& s : sh) {
      if (!s.used) continue;
      for (uint32_t m = 0; m < matCount; ++m)
        if (((s.matSeen >> m) & 1ull) && !seen[m]) { seen[m] = true; stack.push_back(m); }
    }
    // spawns may add any row: be conservative once a scene exists
    while (!stack.empty()) {
      uint32_t m = stack.back();
      stack.pop_back();
      for (int f : {M_meltTo, M_freezeTo, M_boilTo, M_condTo, M_burnTo, M_splitTo, M_corrTo}) {
        uint32_t t = (uint32_t)row(m)[f];
        if (t < matCount && !seen[t]) { seen[t] = true; stack.push_back(t); }
      }
    }
    bool fr = false, bo = false, se = false;
    for (uint32_t m = 0; m < matCount; ++m) {
      if (!seen[m]) continue;
      if (row(m)[M_fric] != 0 || row(m)[M_bondK] != 0) fr = true;
      if (row(m)[M_bondK] != 0) bo = true;
      if (seal_row(m)) se = true;
    }
    if (fr != hasFriction || bo != hasBonds || se != hasSeal) graphValid = false;
    hasFriction = fr;
    hasBonds = bo;
    hasSeal = se;
  }

  // Recompute the colour-major key layout over the active scenes.
  // The clocks in ScenePar (formClock, bondDirty, formNow, substep) advance on
  // the device; before the host pushes the whole parameter array again (scene
  // added or removed) it takes them back, except for a scene whose parameters
  // the host has just written (freshScene).
  uint32_t freshScene = 0xffffffffu;
  bool paramsStale = false;
  bool merge_device_clocks() {
    if (!paramsStale) return true;
    std::vector<ScenePar> dev(maxScenes);
    if (!cuda_ok(cudaMemcpyAsync(dev.data(), b.scenes, sizeof(ScenePar) * maxScenes, cudaMemcpyDeviceToHost, st),
                 "clocks") ||
        !cuda_ok(cudaStreamSynchronize(st), "clocks"))
      return false;
    for (uint32_t s = 0; s < maxScenes; ++s) {
      if (s == freshScene || !sh[s].used || !sh[s].loaded) continue;
      hpar[s].formClock = dev[s].formClock;
      hpar[s].bondDirty = dev[s].bondDirty;
      hpar[s].formNow = dev[s].formNow;
      hpar[s].substep = dev[s].substep;
    }
    paramsStale = false;
    return true;
  }

  bool relayout() {
    if (!merge_device_clocks()) return false;
    uint32_t slotEnd = 0, nAct = 0, numScenes = 0;
    uint64_t cells = 0;
    for (uint32_t s = 0; s < maxScenes; ++s) {
      SceneHost& h = sh[s];
      if (!h.used) continue;
      slotEnd = std::max(slotEnd, h.slotBase + h.cap);
      if (h.loaded) {
        nAct += h.n;
        cells += (uint64_t)h.gridW * h.gridH;
      }
    }
    if (cells > maxCells) return fail("total grid cells %llu exceed max_cells %u", (unsigned long long)cells, maxCells);
    uint64_t K = 0, tiles = 0;
    tileHost.clear();
    if (!staged) {
      // colour-major layout: every scene's colour-c cells, colour by colour
      uint32_t counts[4] = {0, 0, 0, 0};
      for (uint32_t s = 0; s < maxScenes; ++s) {
        SceneHost& h = sh[s];
        ScenePar& p = hpar[s];
        if (!h.used) { p.active = 0; continue; }
        numScenes = s + 1;
        if (!h.loaded) { p.active = 0; continue; }
        p.tileShift = 0;
        for (int c = 0; c < 4; ++c) {
          const uint32_t nA = (h.gridW + 1 - (c & 1)) / 2;
          const uint32_t nB = (h.gridH + 1 - (c >> 1)) / 2;
          p.keyOff[c] = counts[c];  // relative for now
          p.nA[c] = nA;
          counts[c] += nA * nB;
        }
      }
      uint32_t base[5];
      base[0] = 0;
      for (int c = 0; c < 4; ++c) base[c + 1] = base[c] + counts[c];
      for (uint32_t s = 0; s < maxScenes; ++s)
        if (sh[s].used && sh[s].loaded)
          for (int c = 0; c < 4; ++c) hpar[s].keyOff[c] += base[c];
      for (int c = 0; c < 5; ++c) hw.colourBase[c] = base[c];
      K = base[4];
    } else {
      // tile-major layout, tiles of 4 x 4 cells: at the densities the solver
      // reaches (16 to ~30 particles per 4 wu cell) a tile's neighbourhood of
      // 36 cells stays inside the staging capacity, where 8 x 8 tiles
      // (100 cells) overflow it
      const uint32_t ts = tileShiftPinned ? tileShiftPinned : 2u, T = 1u << ts;
      for (uint32_t s = 0; s < maxScenes; ++s) {
        SceneHost& h = sh[s];
        ScenePar& p = hpar[s];
        if (!h.used) { p.active = 0; continue; }
        numScenes = s + 1;
        if (!h.loaded) { p.active = 0; continue; }
        p.tileShift = ts;
        p.tilesX = (h.gridW + T - 1) >> ts;
        p.tilesY = (h.gridH + T - 1) >> ts;
        p.keyBase = (uint32_t)K;
        p.tileBase = (uint32_t)tiles;
        for (uint32_t ty = 0; ty < p.tilesY; ++ty)
          for (uint32_t tx = 0; tx < p.tilesX; ++tx)
            tileHost.push_back(TileInfo{s, tx, ty, (uint32_t)(K + (((uint64_t)ty * p.tilesX + tx) << (2u * ts)))});
        K += ((uint64_t)p.tilesX * p.tilesY) << (2u * ts);
        tiles += (uint64_t)p.tilesX * p.tilesY;
      }
      for (int c = 0; c < 5; ++c) hw.colourBase[c] = 0;
    }
    if (K >= 0xffffffffull) return fail("grid keys overflow");
    if (!ensure_tile_buffers((uint32_t)K, (uint32_t)tiles)) return false;
    hw.numScenes = numScenes;
    hw.K = (uint32_t)K;
    hw.nTiles = (uint32_t)tiles;
    hw.stageCap = STAGE_MAX;
    hw.slotEnd = slotEnd;
    hw.nAct = nAct;
    update_features();
    default_lanes();
    hw.hasFriction = hasFriction;
    hw.hasBonds = hasBonds;
    layoutDirty = false;
    graphValid = false;
    bool ok = cuda_ok(cudaMemcpyAsync(b.world, &hw, sizeof(hw), cudaMemcpyHostToDevice, st), "world") &&
              cuda_ok(cudaMemcpyAsync(b.scenes, hpar.data(), sizeof(ScenePar) * maxScenes,
                                      cudaMemcpyHostToDevice, st), "scenes");
    return ok && cuda_ok(cudaStreamSynchronize(st), "relayout");
  }

  // Grow the key- and tile-sized buffers to the layout's needs (cell starts
  // of every key, the tile table and the per-substep run table), and upload
  // the tile table.
  std::vector<TileInfo> tileHost;
  uint32_t keyCap = 0, tileCap = 0;
  uint32_t tileShiftPinned = 0;  // the staged layout's tile side, log2 (0: 2, tiles of 4 x 4 cells)
  // the tile-major layout with shared-memory staged gathers (sn_set_staged);
  // off by default: measured slower than the list gathers it replaces
  bool staged = false;
  // the solver iterations as one persistent cooperative kernel (sn_set_persistent); off by default
  bool persistent = false;
  bool ensure_tile_buffers(uint32_t K, uint32_t tiles) {
    if (K + 1 > keyCap) {
      if (b.cellStart) cudaFree(b.cellStart);
      if (b.CB) cudaFree(b.CB);
      keyCap = std::max<uint32_t>(K + 1, keyCap + keyCap / 2);
      b.cellStart = dalloc<uint32_t>(keyCap, err);
      b.CB = dalloc<int4>(keyCap, err);
      if (!b.cellStart || !b.CB) return false;
    }
    if (tiles > tileCap || !b.tiles) {
      if (b.tiles) cudaFree(const_cast<TileInfo*>(b.tiles));
      if (b.TR) cudaFree(b.TR);
      if (b.OVF) cudaFree(b.OVF);
      tileCap = std::max<uint32_t>(std::max<uint32_t>(tiles, 1u), tileCap + tileCap / 2);
      b.tiles = dalloc<TileInfo>(tileCap, err);
      b.TR = dalloc<uint32_t>((size_t)tileCap * TR_STRIDE, err);
      b.OVF = dalloc<uint32_t>(tileCap, err);
      if (!b.tiles || !b.TR || !b.OVF) return false;
    }
    if (!tileHost.empty() &&
        !cuda_ok(cudaMemcpyAsync(const_cast<TileInfo*>(b.tiles), tileHost.data(), sizeof(TileInfo) * tileHost.size(),
                                 cudaMemcpyHostToDevice, st), "tiles"))
      return false;
    return true;
  }

  // Fetch the device-side scene parameters (clocks move on the device).
  bool pull_params() {
    if (!cuda_ok(cudaMemcpyAsync(hpar.data(), b.scenes, sizeof(ScenePar) * maxScenes, cudaMemcpyDeviceToHost, st),
                 "pull"))
      return false;
    if (!cuda_ok(cudaStreamSynchronize(st), "pull")) return false;
    paramsStale = false;
    return true;
  }
  bool push_scene(uint32_t s) {
    return cuda_ok(cudaMemcpyAsync(b.scenes + s, &hpar[s], sizeof(ScenePar), cudaMemcpyHostToDevice, st), "push");
  }

  bool validate_header(const sn_scene* sc, uint32_t cap) {
    if (!sc) return fail("scene is NULL");
    if (sc->n_fluid > sc->n) return fail("scene.nFluid out of range");
    if (sc->n > cap) return fail("scene.n = %u exceeds maxParticles = %u", sc->n, cap);
    if (sc->n > 0 && (!sc->pos || !sc->vel || !sc->mat_id)) return fail("scene arrays missing");
    if (sc->cell_shift < 1 || sc->cell_shift > 27) return fail("cellShift outside 1..27");
    if ((1u << sc->cell_shift) < (uint32_t)KERNEL_H) return fail("cells smaller than the kernel radius");
    if (sc->dom_w < 2 * 32768 || sc->dom_h < 2 * 32768) return fail("domain smaller than the wall margin");
    return true;
  }
  // The per-particle checks of loadScene (src/engine.js:3704-3760), in this
  // order, for particle i; false with the message of the first that fails.
  // k_load_check applies the same tests to every particle on the device.
  bool validate_particle(const sn_scene* sc, uint32_t i) {
    if (sc->mat_id[i] >= matCount) return fail("matId[%u] = %u >= matCount %u", i, sc->mat_id[i], matCount);
    int32_t lo = i < sc->n_fluid ? 0 : -MAX_POS;
    if (sc->pos[2 * i] < lo || sc->pos[2 * i] > MAX_POS || sc->pos[2 * i + 1] < lo || sc->pos[2 * i + 1] > MAX_POS)
      return fail("pos[%u] outside [%d, 2^27]", i, lo);
    if (sc->flags && (sc->flags[i] & ~FLAG_MASK)) return fail("flags[%u] sets a reserved bit", i);
    if (sc->temp && (sc->temp[i] < TEMP_MIN || sc->temp[i] > TEMP_MAX)) return fail("temp[%u] out of range", i);
    if (sc->fuel && sc->fuel[i] < 0) return fail("fuel[%u] < 0", i);
    uint32_t want = row(sc->mat_id[i])[M_phantom] != 0 ? FLAG_DEAD : 0u;
    if (sc->flags && (sc->flags[i] & FLAG_DEAD) && !want) return fail("flags[%u] sets FLAG_DEAD on a live row", i);
    return true;
  }

  // The scene's arrays uploaded as they are (SoA, 8 words per particle:
  // pos 2n, vel 2n, mat n, flags n, temp n, fuel n), checked and packed on
  // the device: a host loop over a 10^6-particle scene costs milliseconds.
  int32_t* upl = nullptr;
  int2* initPos = nullptr;     // [cap] each scene's positions at its last load
  uint32_t* uplRes = nullptr;  // [4]: first failing index, material mask (2 words)
  bool upload_scene(const sn_scene* sc, LoadTables& T, uint64_t* seen) {
    const size_t n = sc->n;
    if (!upl) {
      upl = dalloc<int32_t>((size_t)capSlots * 8, err);
      uplRes = dalloc<uint32_t>(4, err);
      if (!upl || !uplRes) return false;
    }
    bool ok = true;
    auto up = [&](size_t off, const void* src, size_t words) {
      if (src && words) ok = ok && cuda_ok(cudaMemcpyAsync(upl + off, src, words * 4, cudaMemcpyHostToDevice, st), "upload");
    };
    up(0, sc->pos, 2 * n);
    up(2 * n, sc->vel, 2 * n);
    up(4 * n, sc->mat_id, n);
    up(5 * n, sc->flags, n);
    up(6 * n, sc->temp, n);
    up(7 * n, sc->fuel, n);
    const uint32_t init[4] = {0xffffffffu, 0u, 0u, 0u};
    ok = ok && cuda_ok(cudaMemcpyAsync(uplRes, init, 16, cudaMemcpyHostToDevice, st), "upload");
    if (!ok) return false;
    const uint32_t present = (sc->flags ? 1u : 0u) | (sc->temp ? 2u : 0u) | (sc->fuel ? 4u : 0u);
    if (n) k_load_check<<<grid_for(n), 256, 0, st>>>(upl, sc->n, sc->n_fluid, matCount, present, T, uplRes);
    uint32_t res[4];
    cudaMemcpyAsync(res, uplRes, 16, cudaMemcpyDeviceToHost, st);
    if (!cuda_ok(cudaStreamSynchronize(st), "load check")) return false;
    if (res[0] != 0xffffffffu) {
      if (!validate_particle(sc, res[0])) return false;
      return fail("particle %u failed the device check but passes the host check", res[0]);
    }
    *seen = (uint64_t)res[1] | ((uint64_t)res[2] << 32);
    return true;
  }

  // loadScene packing (src/engine.js:3704-3951) into scene s.
  bool load(uint32_t s, const sn_scene* sc) {
    accFresh = false;
    sortedFresh = false;
    SceneHost& h = sh[s];
    if (!validate_header(sc, h.cap)) return false;
    LoadTables T;
    for (uint32_t m = 0; m < MAT_MAX; ++m) {
      if (m >= matCount) { T.fluidFl[m] = T.wallFl[m] = 0u; T.fuel0[m] = 0; continue; }
      const int32_t* r = row(m);
      T.wallFl[m] = (r[M_phantom] != 0 ? FLAG_DEAD : 0u) | (seal_row(m) ? FLAG_SEAL : 0u);
      T.fluidFl[m] = T.wallFl[m] | (spawn_welds(m) ? (1u << 8) : 0u);
      T.fuel0[m] = r[M_fuel0];
    }
    uint64_t seenMask = 0;
    if (!upload_scene(sc, T, &seenMask)) return false;
    // loadScene's copy of the loaded positions (_initialPos, src/engine.js:3947),
    // kept on the device for liveness
    if (!initPos) {
      initPos = dalloc<int2>(capSlots, err);
      if (!initPos) return false;
    }
    if (sc->n && !cuda_ok(cudaMemcpyAsync(initPos + h.slotBase, upl, (size_t)sc->n * 8, cudaMemcpyDeviceToDevice, st),
                          "initial positions"))
      return false;
    h.nInit = sc->n;
    // a scene load dissolves every body of the scene (src/engine.js:3811-3813)
    if (!drop_scene_bodies(s)) return false;
    uint32_t cs = 1u << sc->cell_shift;
    uint32_t gW = std::max<uint32_t>(1, (uint32_t)(((int64_t)sc->dom_w + cs - 1) / cs));
    uint32_t gH = std::max<uint32_t>(1, (uint32_t)(((int64_t)sc->dom_h + cs - 1) / cs));
    h.n = sc->n;
    h.nFluid = sc->n_fluid;
    h.gridW = gW;
    h.gridH = gH;
    h.cellShift = sc->cell_shift;
    h.cellTotal = gW * gH;
    h.domW = sc->dom_w;
    h.domH = sc->dom_h;
    h.substeps = 0;
    h.nFluid0 = sc->n_fluid;
    const size_t nf = sc->n_fluid, nn = sc->n;
    h.bpos.assign(sc->pos + 2 * nf, sc->pos + 2 * nn);
    h.bmat.assign(sc->mat_id + nf, sc->mat_id + nn);
    h.hasTemp = sc->temp != nullptr;
    h.hasFuel = sc->fuel != nullptr;
    h.btemp.assign(nn - nf, 0);
    h.bfuel.assign(nn - nf, 0);
    if (sc->temp) h.btemp.assign(sc->temp + nf, sc->temp + nn);
    if (sc->fuel) h.bfuel.assign(sc->fuel + nf, sc->fuel + nn);
    h.weldSeq = 1;
    h.weldHold = h.weldHoldSeq = h.fuseTag = h.lastWeldTag = 0;
    h.wallsOn = true;
    h.events.clear();
    h.consumed = 0;
    eventsDirty = true;
    h.matSeen = seenMask;
    k_load_pack<<<grid_for(h.cap), 256, 0, st>>>(upl, sc->n, sc->n_fluid, h.cap,
                                                  (sc->flags ? 1u : 0u) | (sc->temp ? 2u : 0u) | (sc->fuel ? 4u : 0u), T,
                                                  b.state + (size_t)h.slotBase * 8);
    bool ok = cuda_ok(cudaGetLastError(), "pack") &&
              cuda_ok(cudaMemsetAsync(b.stacc + h.slotBase, 0, sizeof(int2) * h.cap, st), "stacc") &&
              cuda_ok(cudaMemsetAsync(b.bond + (size_t)h.slotBase * BOND_CAP, 0, 4ull * BOND_CAP * h.cap, st), "bond") &&
              cuda_ok(cudaMemsetAsync(b.bondCand + (size_t)h.slotBase * BOND_CAP, 0, 4ull * BOND_CAP * h.cap, st),
                      "bondCand");
    if (ok) {
      k_fill_u32<<<grid_for(h.cap), 256, 0, st>>>(b.sceneOf + h.slotBase, h.cap, s);
      ok = cuda_ok(cudaGetLastError(), "sceneOf");
    }
    if (!ok) return false;
    ScenePar& p = hpar[s];
    p = ScenePar{};
    p.slotBase = h.slotBase;
    p.cap = h.cap;
    p.n = h.n;
    p.nFluid = h.nFluid;
    p.gridW = gW;
    p.gridH = gH;
    p.cellShift = h.cellShift;
    p.cellTotal = h.cellTotal;
    p.domW = h.domW;
    p.domH = h.domH;
    p.vmax = VMAX;
    p.weldHold = 0;
    p.formClock = 0;
    p.bondDirty = 1;
    p.formNow = 0;
    p.active = 1;
    h.loaded = true;
    if (!reset_chain(s)) return false;
    uint32_t zero8[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    cudaMemcpyAsync(b.acc + s * 8, zero8, 32, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(b.accLast + s * 8, zero8, 32, cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(b.dbg, 0, 64, st);
    cudaMemsetAsync(b.err, 0, 16, st);
    freshScene = s;
    bool ok2 = relayout();
    freshScene = 0xffffffffu;
    return ok2;
  }

  bool reset_chain(uint32_t s) {
    static const uint32_t CHAIN_INIT[8] = {0x243f6a88u, 0x85a308d3u, 0x13198a2eu, 0x03707344u,
                                           0xa4093822u, 0x299f31d0u, 0x082efa98u, 0xec4e6c89u};
    return cuda_ok(cudaMemcpyAsync(b.chain + s * 8, CHAIN_INIT, 32, cudaMemcpyHostToDevice, st), "chain");
  }

  // Resident CTAs per SM of a kernel at 256 threads (cached per kernel); a
  // grid of numSMs x that runs in one wave and grid-strides over its items.
  std::vector<std::pair<const void*, int>> occCache;
  int occ_blocks(const void* k) {
    for (auto& kv : occCache)
      if (kv.first == k) return kv.second;
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, 256, 0) != cudaSuccess || nb < 1) nb = 1;
    occCache.push_back({k, nb});
    return nb;
  }
  int grid_occ(const void* k, uint64_t items) {
    uint64_t g = (items + 255) / 256;
    uint64_t cap = (uint64_t)numSMs * occ_blocks(k);
    return (int)std::max<uint64_t>(1, std::min(g, cap));
  }

  int grid_for(uint64_t items) const {
    uint64_t g = (items + 255) / 256;
    uint64_t cap = (uint64_t)numSMs * 8;
    if (g > cap) g = cap;
    return (int)std::max<uint64_t>(g, 1);
  }

  // Optional phase markers (profile_substep): events recorded between phases.
  cudaEvent_t* pev = nullptr;
  int npev = 0;
  void mark() {
    if (pev) cudaEventRecord(pev[npev++], st);
  }

  // Lanes per particle for the neighbour gathers: small scenes split each
  // neighbour list over several lanes so the GPU has enough threads in flight.
  // Lanes per particle for each gather class (solveA, the colour passes,
  // post1, post2). Results do not depend on them (split sums are exact); only
  // speed does, so the autotuner may try them on real substeps.
  struct LaneCfg {
    int a = 1, c = 1, p1 = 1, p2 = 1, n = 1;
  };
  LaneCfg lanesCfg, pinnedLanes;
  bool autoLanes = true, lanesTuned = false, setLanes = false;
  uint32_t tunedAtN = 0;

  // The tile-staged kernels: one CTA per tile, at most as many CTAs as fit
  // on the GPU at once (grid-stride over the tiles beyond that).
  size_t stage_bytes() const { return (size_t)hw.stageCap * sizeof(int4); }
  int grid_tiles(const void* fn) {
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, 256, stage_bytes());
    const uint64_t cap = (uint64_t)numSMs * (uint64_t)std::max(per, 1);
    // at least two CTAs per SM, for the tiles too large to stage, which the
    // whole grid shares
    return (int)std::min<uint64_t>(cap, std::max<uint64_t>(hw.nTiles, 2ull * numSMs));
  }
  template <bool DBG, int L>
  void launch_solveA(int lastIter) {
    if (staged)
      k_solveA_tiled<DBG, L><<<grid_tiles((const void*)k_solveA_tiled<DBG, L>), 256, stage_bytes(), st>>>(b, lastIter);
    else
      k_solveA<DBG, L><<<grid_occ((const void*)k_solveA<DBG, L>, (uint64_t)hw.nAct * L), 256, 0, st>>>(b, lastIter);
  }
  template <bool DBG, int L>
  void launch_colours() {
    if (staged) {
      const int g = grid_tiles((const void*)k_colour_tiled<DBG, L, false>);
      k_colour_tiled<DBG, L, true><<<g, 256, stage_bytes(), st>>>(b, 0, b.PL, b.PL2);
      k_colour_tiled<DBG, L, false><<<g, 256, stage_bytes(), st>>>(b, 1, b.PL2, b.PL);
      k_colour_tiled<DBG, L, false><<<g, 256, stage_bytes(), st>>>(b, 2, b.PL, b.PL2);
      k_colour_tiled<DBG, L, false><<<g, 256, stage_bytes(), st>>>(b, 3, b.PL2, b.PL);
      return;
    }
    const int g = grid_occ((const void*)k_colour<DBG, L>, (uint64_t)hw.nAct * L / 4 + 256);
    for (int c = 0; c < 4; ++c) {
      const int4* src = (c & 1) ? b.PL2 : b.PL;
      int4* dst = (c & 1) ? b.PL : b.PL2;
      cudaEventRecord(evFork, st);
      cudaStreamWaitEvent(st2, evFork, 0);
      k_colour_copy<<<2 * numSMs, 256, 0, st2>>>(b, c, src, dst);
      cudaEventRecord(evJoin, st2);
      k_colour<DBG, L><<<g, 256, 0, st>>>(b, c, src, dst, 0);
      cudaStreamWaitEvent(st, evJoin, 0);
    }
  }
  // One cooperative launch of every solver iteration (k_iters_persistent):
  // the grid is exactly the resident capacity, which the cooperative launch
  // guarantees to run at once (its grid barriers need every CTA resident).
  uint32_t* barBuf = nullptr;
  template <bool DBG, int L>
  void launch_persistent() {
    const void* fn = (const void*)k_iters_persistent<DBG, L>;
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, 256, 0);
    cudaMemsetAsync(barBuf, 0, 8, st);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(std::max(per, 1) * numSMs));
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k_iters_persistent<DBG, L>, b, iters, barBuf);
  }
  template <bool DBG, int L>
  void launch_contain_stress() {
    k_contain_stress<DBG, L>
        <<<grid_occ((const void*)k_contain_stress<DBG, L>, (uint64_t)hw.slotEnd * L), 256, 0, st>>>(b);
  }
  // friction splits each list like the colour passes and takes their lanes
  template <bool DBG, int L>
  void launch_friction() {
    k_friction<DBG, L><<<grid_occ((const void*)k_friction<DBG, L>, (uint64_t)hw.nAct * L), 256, 0, st>>>(b);
  }
  template <bool DBG, int L>
  void launch_nbr() {
    if (staged)
      k_nbr<DBG, L, true><<<grid_occ((const void*)k_nbr<DBG, L, true>, (uint64_t)hw.nAct * L), 256, 0, st>>>(b);
    else
      k_nbr<DBG, L, false><<<grid_occ((const void*)k_nbr<DBG, L, false>, (uint64_t)hw.nAct * L), 256, 0, st>>>(b);
  }
  template <bool DBG, int L>
  void launch_post1() {
    k_post1<DBG, L><<<grid_occ((const void*)k_post1<DBG, L>, (uint64_t)hw.nAct * L), 256, 0, st>>>(b);
  }
  template <bool DBG, bool HASH, int L>
  void launch_post2(int formFlags) {
    k_post2<DBG, HASH, L><<<grid_occ((const void*)k_post2<DBG, HASH, L>, (uint64_t)hw.nAct * L), 256, 0, st>>>(
        b, formFlags);
  }
#define SN_LANES(LV, CALL)      \
  switch (LV) {                 \
    case 8: { constexpr int L_ = 8; CALL; } break; \
    case 4: { constexpr int L_ = 4; CALL; } break; \
    case 2: { constexpr int L_ = 2; CALL; } break; \
    default: { constexpr int L_ = 1; CALL; } break; \
  }

  template <bool DBG>
  void launch_substep() {
    const LaneCfg lc = lanesCfg;
    const int gs = grid_for(hw.slotEnd);
    const int ga = grid_for(hw.nAct);
    uint64_t Lc = 0;
    if (anyEvents) {
      k_impulse_sched<<<hw.numScenes, IMPULSE_THREADS, 0, st>>>(b, devEv, devEp);
      ++Lc;
    }
    mark();
    k_predict_key<DBG><<<gs, 256, 0, st>>>(b);
    ++Lc;
    // §20: rigidStep runs before predict in the reference; predict leaves
    // members at pred = pos, so placing them after it is the same substep.
    const uint32_t nB = (uint32_t)bodies.size();
    if (nB) {
      k_rigid_step<DBG><<<nB, RG_THREADS, 0, st>>>(b);
      ++Lc;
    }
    mark();
    int bits = 1;
    while ((1ull << bits) <= hw.K) ++bits;
    radix::sort_pairs(b.keys, hw.slotEnd, bits, b.skey, b.sslot, tmpK, tmpV, hist, st);
    Lc += (uint64_t)radix::LAUNCHES_PER_PASS * ((bits + radix::RBITS - 1) / radix::RBITS);
    mark();
    // the cell ranges (from the sorted keys) and the gather (from the sorted
    // slots) share no word: the ranges run on the side branch
    cudaEventRecord(evFork, st);
    cudaStreamWaitEvent(st2, evFork, 0);
    k_cellstart<<<grid_for((uint64_t)hw.K + 1), 256, 0, st2>>>(b);
    cudaEventRecord(evJoin, st2);
    k_gather<<<ga, 256, 0, st>>>(b);
    cudaStreamWaitEvent(st, evJoin, 0);
    if (staged) k_tiles<<<grid_for((uint64_t)hw.nTiles * 32), 256, 0, st>>>(b);
    if (!DBG) {
      k_cellbox<<<grid_for((uint64_t)hw.K * 32), 256, 0, st>>>(b, boxChunks);
      k_cellbox_chunks<<<numSMs * 2, 256, 0, st>>>(b, boxChunks);
    }
    mark();
    SN_LANES(lc.n, (launch_nbr<DBG, L_>()));
    mark();
    Lc += 3 + (staged ? 1 : 0) + (DBG ? 0 : 2);
    // the persistent form of the iteration loop (sn_set_persistent): worlds
    // with no rigid body, in the colour-major layout, and not while
    // profile_substep times the phases one by one
    const bool persist = persistent && !staged && nB == 0 && pev == nullptr;
    if (persist) {
      SN_LANES(lc.c, (launch_persistent<DBG, L_>()));
      Lc += 1;
    }
    for (uint32_t it = 0; it < (persist ? 0u : iters); ++it) {
      const int last = it + 1 == iters ? 1 : 0;
      SN_LANES(lc.a, (launch_solveA<DBG, L_>(last)));
      mark();
      SN_LANES(lc.c, (launch_colours<DBG, L_>()));
      mark();
      Lc += staged ? 5 : 9;
      if (hasFriction) {
        SN_LANES(lc.c, (launch_friction<DBG, L_>()));
        k_apply_fric<DBG><<<ga, 256, 0, st>>>(b);
        Lc += 2;
      }
      if (nB) {
        k_rigid_solve<DBG><<<nB, RG_THREADS, 0, st>>>(b, hasSeal ? 1 : 0);
        ++Lc;
      }
      mark();
    }
    if (hasSeal) {
      k_contain<DBG><<<grid_for(hw.nAct), 256, 0, st>>>(b);
      ++Lc;
    }
    SN_LANES(lc.p1, (launch_post1<DBG, L_>()));
    ++Lc;
    mark();
    if (hasBonds || nB) {
      SN_LANES(lc.p2, (launch_post2<DBG, false, L_>(0)));
      if (hasSeal) {
        // the members of seal bodies walk their lists: split them like friction
        SN_LANES(nB ? lc.c : 1, (launch_contain_stress<DBG, L_>()));
        ++Lc;
      }
      if (nB) {
        k_rigid_member<DBG><<<nB, RG_THREADS, 0, st>>>(b);
        ++Lc;
      }
      k_form1<DBG><<<ga, 256, 0, st>>>(b);
      if (chainOn) k_form2<true><<<gs, 256, 0, st>>>(b, b.acc);
      else k_form2<false><<<gs, 256, 0, st>>>(b, nullptr);
      Lc += 3;
    } else if (chainOn) {
      SN_LANES(lc.p2, (launch_post2<DBG, true, L_>(1)));
      ++Lc;
    } else {
      SN_LANES(lc.p2, (launch_post2<DBG, false, L_>(1)));
      ++Lc;
    }
    mark();
    k_fold<<<(hw.numScenes + 63) / 64, 64, 0, st>>>(b, chainOn ? 1 : 0);
    ++Lc;
    mark();
    launchesPerSubstep = Lc;
  }
#undef SN_LANES

  // Lanes before (or without) tuning, from the active particle count: each
  // class is sized by the particles one launch works on and how heavy its
  // per-particle epilogue is (measured on the 1 M-particle scene: solveA 1,
  // colours 4, post1 2, post2 1).
  static int lanes_for(uint64_t n) {
    if (n < 40000) return 8;
    if (n < 80000) return 4;
    if (n < 160000) return 2;
    return 1;
  }
  void default_lanes() {
    if (!autoLanes) {
      lanesCfg = setLanes ? pinnedLanes
                          : LaneCfg{lanesOverride, lanesOverride, lanesOverride, lanesOverride, lanesOverride};
      return;
    }
    if (lanesTuned && hw.nAct * 2 >= tunedAtN && hw.nAct <= tunedAtN * 2ull) return;
    lanesTuned = false;
    const uint64_t n = hw.nAct;
    lanesCfg = LaneCfg{lanes_for(n), lanes_for(n / 16), lanes_for(n / 8), lanes_for(n), lanes_for(n)};
  }

  // The autotuner: run `per` real substeps under each uniform lane count with
  // phase events, then keep the fastest count per gather class. Every lane
  // count gives the same results, so the tuning substeps are ordinary
  // substeps of the scenes (they count toward the caller's request).
  // Pin the lanes of every gather class (e.g. ones tuned on another run of
  // the same workload); the size rule and the tuner stop changing them.
  bool set_lanes(const uint32_t* v) {
    if (!v) return fail("lanes are NULL");
    for (int k = 0; k < 5; ++k)
      if (v[k] != 1 && v[k] != 2 && v[k] != 4 && v[k] != 8) return fail("lanes must be 1, 2, 4 or 8");
    lanesCfg = LaneCfg{(int)v[0], (int)v[1], (int)v[2], (int)v[3], (int)v[4]};
    pinnedLanes = lanesCfg;
    setLanes = true;
    autoLanes = false;
    lanesTuned = true;
    graphValid = false;
    return true;
  }

  bool autotune(uint32_t per, uint32_t* used) {
    if (used) *used = 0;
    if (!autoLanes) return true;  // lanes were pinned at create
    bool any = false;
    for (auto& s2 : sh) any |= (s2.used && s2.loaded);
    if (!any) return fail("autotune before loadScene()");
    if (layoutDirty && !relayout()) return false;
    if (eventsDirty && !upload_events()) return false;
    return tune_lanes(std::max(1u, per), used);
  }

  // Layout tuning: the list gathers (colour-major keys) and the tile-staged
  // gathers with tiles of 4, 8 and 16 cells, each run for one untimed
  // substep (it re-lays out and re-captures) and `per` timed ones; the
  // fastest stays. Every layout gives the same results, so these are the
  // scenes' real substeps. ms[k] = device ms per substep of candidate k.
  bool autotune_layout(uint32_t per, uint32_t* used, uint32_t* pick, float* ms) {
    static const uint32_t cand[4] = {0u, 2u, 3u, 4u};
    if (used) *used = 0;
    bool any = false;
    for (auto& s2 : sh) any |= (s2.used && s2.loaded);
    if (!any) return fail("autotune before loadScene()");
    per = std::max(1u, per);
    float best = 0.f;
    uint32_t bestC = 0, n = 0;
    for (int ci = 0; ci < 4; ++ci) {
      staged = cand[ci] != 0u;
      if (staged) tileShiftPinned = cand[ci];
      layoutDirty = true;
      if (!step(1) || !step(per)) return false;
      n += per + 1;
      float t = 0.f;
      if (!timing(&t)) return false;
      t /= (float)per;
      if (ms) ms[ci] = t;
      if (ci == 0 || t < best) {
        best = t;
        bestC = cand[ci];
      }
    }
    staged = bestC != 0u;
    if (staged) tileShiftPinned = bestC;
    layoutDirty = true;
    if (used) *used = n;
    if (pick) *pick = bestC;
    return true;
  }

  bool tune_lanes(uint32_t per, uint32_t* used) {
    static const int cand[4] = {1, 2, 4, 8};
    const int NE = 8 + 3 * (int)iters + 4;
    std::vector<cudaEvent_t> evs(NE);
    for (auto& e : evs) cudaEventCreate(&e);
    double best[5] = {1e30, 1e30, 1e30, 1e30, 1e30};
    int pick[5] = {1, 1, 1, 1, 1};
    uint32_t n = 0;
    bool ok = true;
    for (int ci = 0; ci < 4 && ok; ++ci) {
      lanesCfg = LaneCfg{cand[ci], cand[ci], cand[ci], cand[ci], cand[ci]};
      double t[5] = {0, 0, 0, 0, 0};
      // rep 0 is untimed: a kernel's first launch also loads its module
      for (uint32_t r = 0; r <= per && ok; ++r) {
        pev = r > 0 ? evs.data() : nullptr;
        npev = 0;
        launch_one();
        int used2 = npev;
        pev = nullptr;
        ok = cuda_ok(cudaStreamSynchronize(st), "tune");
        for (auto& s2 : sh)
          if (s2.used && s2.loaded) s2.substeps += 1;
        paramsStale = true;
        accFresh = chainOn;
        ++n;
        if (r == 0) continue;
        auto span = [&](int k) {
          float ms = 0.f;
          if (k + 1 < used2) cudaEventElapsedTime(&ms, evs[k], evs[k + 1]);
          return (double)ms;
        };
        // phases: 0 predict, 1 sort, 2 ranges+gather, 3 nbr, then per
        // iteration (solveA, colours, friction), then post1, post2, fold
        for (uint32_t it = 0; it < iters; ++it) {
          t[0] += span(4 + 3 * (int)it);
          t[1] += span(5 + 3 * (int)it);
        }
        t[2] += span(4 + 3 * (int)iters);
        t[3] += span(5 + 3 * (int)iters);
        t[4] += span(3);
      }
      for (int k = 0; k < 5; ++k)
        if (t[k] < best[k]) {
          best[k] = t[k];
          pick[k] = cand[ci];
        }
    }
    for (auto& e : evs) cudaEventDestroy(e);
    lanesCfg = LaneCfg{pick[0], pick[1], pick[2], pick[3], pick[4]};
    lanesTuned = true;
    tunedAtN = hw.nAct;
    graphValid = false;
    if (used) *used = n;
    return ok;
  }

  void launch_one() {
    if (debug) launch_substep<true>();
    else launch_substep<false>();
  }

  bool upload_events() {
    std::vector<ImpulseEv> all;
    std::vector<EvPar> ep(maxScenes, EvPar{0, 0, 0, 0});
    anyEvents = false;
    for (uint32_t s = 0; s < maxScenes; ++s) {
      SceneHost& h = sh[s];
      ep[s].begin = (uint32_t)all.size();
      if (h.used && h.loaded) {
        uint32_t consumed = 0;
        for (const ImpulseEv& e : h.events)
          if ((uint64_t)e.at < h.substeps) ++consumed;
        for (const ImpulseEv& e : h.events) all.push_back(e);
        ep[s].cursor = ep[s].begin + consumed;
        if (consumed < h.events.size()) anyEvents = true;
      } else {
        ep[s].cursor = ep[s].begin;
      }
      ep[s].end = (uint32_t)all.size();
    }
    if (all.size() > devEvCap) {
      if (devEv) cudaFree(devEv);
      devEvCap = std::max<size_t>(all.size(), 256);
      devEv = dalloc<ImpulseEv>(devEvCap, err);
      if (!devEv) return false;
    }
    if (!all.empty() &&
        !cuda_ok(cudaMemcpyAsync(devEv, all.data(), all.size() * sizeof(ImpulseEv), cudaMemcpyHostToDevice, st),
                 "events"))
      return false;
    if (!cuda_ok(cudaMemcpyAsync(devEp, ep.data(), ep.size() * sizeof(EvPar), cudaMemcpyHostToDevice, st), "ep"))
      return false;
    eventsDirty = false;
    graphValid = false;
    return true;
  }

  bool step(uint32_t count) {
    if (hw.nAct == 0 && count > 0) {
      bool any = false;
      for (auto& s : sh) any |= (s.used && s.loaded);
      if (!any) return fail("step() called before loadScene()");
    }
    if (count == 0) return true;
    if (layoutDirty && !relayout()) return false;
    if (eventsDirty && !upload_events()) return false;
    if (useGraph && !graphValid) {
      if (gexec) { cudaGraphExecDestroy(gexec); gexec = nullptr; }
      if (graph) { cudaGraphDestroy(graph); graph = nullptr; }
      if (!cuda_ok(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "capture")) return false;
      launch_one();
      if (!cuda_ok(cudaStreamEndCapture(st, &graph), "endCapture")) return false;
      if (!cuda_ok(cudaGraphInstantiate(&gexec, graph, 0), "instantiate")) return false;
      graphValid = true;
    }
    cudaEventRecord(ev0, st);
    for (uint32_t i = 0; i < count; ++i) {
      if (useGraph) {
        if (!cuda_ok(cudaGraphLaunch(gexec, st), "graphLaunch")) return false;
      } else {
        launch_one();
      }
    }
    cudaEventRecord(ev1, st);
    for (auto& s : sh)
      if (s.used && s.loaded) s.substeps += count;
    lastLaunches = launchesPerSubstep * count;
    paramsStale = true;
    accFresh = chainOn;
    sortedFresh = true;
    // step() (src/engine.js:3990-3997): an armed fusion outlives its gesture
    // only until the formation pass after release, i.e. this call.
    for (uint32_t s2 = 0; s2 < maxScenes; ++s2)
      if (sh[s2].used && sh[s2].loaded && sh[s2].fuseTag != 0 && sh[s2].weldHold == 0 && !set_fuse(s2, 0)) return false;
    return cuda_ok(cudaGetLastError(), "step");
  }

  // profileSubstep (src/engine.js:4221-4267): run `reps` substeps outside the
  // graph with events between phases; out[k] = mean device ms of phase k.
  // Phases: 0 predict, 1 sort, 2 cellstart+gather, 3 nbr, then per
  // iteration (solveA, colours, friction), then post1, post2(+formation+hash), fold.
  bool profile(uint32_t reps, float* out, uint32_t maxOut, uint32_t* nOut) {
    if (layoutDirty && !relayout()) return false;
    if (eventsDirty && !upload_events()) return false;
    const int NE = 8 + 3 * (int)iters + 4;
    std::vector<cudaEvent_t> evs(NE);
    for (auto& e : evs) cudaEventCreate(&e);
    std::vector<double> acc(NE, 0.0);
    int used = 0;
    for (uint32_t r = 0; r < reps; ++r) {
      pev = evs.data();
      npev = 0;
      launch_one();
      used = npev;
      pev = nullptr;
      if (!cuda_ok(cudaStreamSynchronize(st), "profile")) return false;
      for (int k = 0; k + 1 < used; ++k) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, evs[k], evs[k + 1]);
        acc[k] += ms;
      }
      for (auto& s2 : sh)
        if (s2.used && s2.loaded) s2.substeps += 1;
      paramsStale = true;
      accFresh = chainOn;
      sortedFresh = true;
    }
    for (auto& e : evs) cudaEventDestroy(e);
    uint32_t n = (uint32_t)std::max(0, used - 1);
    for (uint32_t k = 0; k < n && k < maxOut; ++k) out[k] = (float)(acc[k] / std::max(1u, reps));
    if (nOut) *nOut = n;
    return true;
  }

  bool timing(float* ms) {
    if (!cuda_ok(cudaEventSynchronize(ev1), "timing")) return false;
    cudaEventElapsedTime(ms, ev0, ev1);
    return true;
  }

  // accFresh: the last substep's digest (kept by the fold in accLast) is the
  // digest of the current state, so digest() needs no hashing pass. Any call
  // that changes a scene's state outside a substep clears it.
  bool accFresh = false;
  // sortedFresh: the sorted-space arrays (inv, RX, NBRN, cellStart) still
  // describe the current slots: set by a substep, cleared by every call that
  // changes which particle sits in which slot.
  bool sortedFresh = false;
  bool digest(uint32_t s, uint32_t out[8]) {
    if (accFresh && !layoutDirty) {
      cudaMemcpyAsync(out, b.accLast + s * 8, 32, cudaMemcpyDeviceToHost, st);
      return cuda_ok(cudaStreamSynchronize(st), "digest");
    }
    if (layoutDirty && !relayout()) return false;
    cudaMemsetAsync(accTmp, 0, sizeof(uint32_t) * 8 * maxScenes, st);
    k_hash<<<grid_for(hw.slotEnd), 256, 0, st>>>(b, accTmp);
    cudaMemcpyAsync(out, accTmp + s * 8, 32, cudaMemcpyDeviceToHost, st);
    return cuda_ok(cudaStreamSynchronize(st), "digest");
  }
  bool read_words(const void* dsrc, void* out, size_t bytes) {
    cudaMemcpyAsync(out, dsrc, bytes, cudaMemcpyDeviceToHost, st);
    return cuda_ok(cudaStreamSynchronize(st), "read");
  }

  // readDerived's rho column and readNbrN's counts (src/engine.js:4290-4291)
  // for scene s, slot order; either output may be null.
  bool read_fields(uint32_t s, int32_t* rho, uint32_t* nbr) {
    if (!sortedFresh || layoutDirty) return fail("no substep has run since the particles last changed");
    const SceneHost& h = sh[s];
    if (h.n == 0) return true;
    k_slot_fields<<<grid_for(h.n), 256, 0, st>>>(b, h.slotBase, h.n, h.nFluid, reinterpret_cast<int32_t*>(tmpK),
                                                 tmpV);
    if (rho) cudaMemcpyAsync(rho, tmpK, (size_t)h.n * 4, cudaMemcpyDeviceToHost, st);
    if (nbr) cudaMemcpyAsync(nbr, tmpV, (size_t)h.n * 4, cudaMemcpyDeviceToHost, st);
    return cuda_ok(cudaStreamSynchronize(st), "readFields");
  }

  bool impulse_now(uint32_t s, int32_t cx, int32_t cy, int32_t r, int32_t ix, int32_t iy, uint32_t limit,
                   uint32_t* hitsOut) {
    accFresh = false;
    ImpulseEv ev{0, cx, cy, r, ix, iy, limit, 0};
    k_impulse_now<<<1, 256, 0, st>>>(b, s, ev, hits);
    uint32_t h = 0;
    cudaMemcpyAsync(&h, hits, 4, cudaMemcpyDeviceToHost, st);
    if (!cuda_ok(cudaStreamSynchronize(st), "impulse")) return false;
    if (hitsOut) *hitsOut = h;
    return true;
  }

  // spawnFluid (src/engine.js:5901-6020) for scene s.
  bool spawn(uint32_t s, const sn_particle* list, uint32_t k, bool noWeld, uint32_t* nOut, bool ownGroup = false) {
    accFresh = false;
    sortedFresh = false;
    SceneHost& h = sh[s];
    if (!h.loaded) return fail("spawn before loadScene");
    if (k == 0) { if (nOut) *nOut = h.n; return true; }
    uint32_t nB = h.n - h.nFluid;
    uint32_t newFluid = h.nFluid + k, newN = newFluid + nB;
    if (newN > h.cap) { if (nOut) *nOut = h.n; return true; }
    for (uint32_t i = 0; i < k; ++i) {
      // Positions far outside any domain are refused: every pred difference the
      // solver forms then stays inside i32 (see the range note in sim2d.cuh).
      if (list[i].x < -(1 << 28) || list[i].x > (1 << 28) || list[i].y < -(1 << 28) || list[i].y > (1 << 28))
        return fail("spawn position outside [-2^28, 2^28]");
    }
    // §18.2 W1 + §18.22 (src/engine.js:5925-5935): one gesture is one group;
    // a spawn outside an open gesture is its own group.
    const uint32_t seq = (h.weldHoldSeq != 0 && !ownGroup) ? h.weldHoldSeq : next_weld_seq(s);
    const uint32_t weldTag = (seq << 8) & WELD_TAG_MASK;
    h.lastWeldTag = weldTag;
    uint32_t total = k + nB;
    std::vector<int32_t> stw((size_t)total * 8, 0);
    for (uint32_t i = 0; i < k; ++i) {
      const sn_particle& q = list[i];
      uint32_t m = (uint32_t)std::min<int32_t>((int32_t)matCount - 1, std::max<int32_t>(0, q.mat));
      const int32_t* r = row(m);
      int32_t* w = &stw[(size_t)i * 8];
      w[0] = q.x;
      w[1] = q.y;
      w[2] = q.vx;
      w[3] = q.vy;
      w[4] = (int32_t)m;
      w[5] = (int32_t)((q.flags & SPAWN_FLAG_MASK) | (r[M_phantom] != 0 ? FLAG_DEAD : 0u) |
                       (seal_row(m) ? FLAG_SEAL : 0u) | ((!noWeld && spawn_welds(m)) ? weldTag : 0u));
      int32_t t = q.has_temp ? q.temp : r[M_spawnTemp];
      w[6] = std::max(TEMP_MIN, std::min(TEMP_MAX, t));
      w[7] = std::max(0, q.has_fuel ? q.fuel : r[M_fuel0]);
    }
    for (uint32_t bb = 0; bb < nB; ++bb) {
      int32_t* w = &stw[(size_t)(k + bb) * 8];
      w[0] = h.bpos[2 * bb];
      w[1] = h.bpos[2 * bb + 1];
      w[4] = (int32_t)h.bmat[bb];
      w[6] = h.hasTemp ? h.btemp[bb] : AMBIENT;
      w[7] = h.hasFuel ? h.bfuel[bb] : row(h.bmat[bb])[M_fuel0];
    }
    size_t off = (size_t)h.slotBase + h.nFluid;
    bool ok = cuda_ok(cudaMemcpyAsync(b.state + off * 8, stw.data(), stw.size() * 4, cudaMemcpyHostToDevice, st),
                      "spawn state") &&
              cuda_ok(cudaMemsetAsync(b.stacc + off, 0, sizeof(int2) * total, st), "spawn stacc") &&
              cuda_ok(cudaMemsetAsync(b.bond + off * BOND_CAP, 0, 4ull * BOND_CAP * k, st), "spawn bond") &&
              cuda_ok(cudaMemsetAsync(b.bondCand + off * BOND_CAP, 0, 4ull * BOND_CAP * k, st), "spawn cand");
    if (!ok || !pull_params()) return false;
    h.n = newN;
    h.nFluid = newFluid;
    for (uint32_t i = 0; i < k; ++i)
      h.matSeen |= 1ull << (uint32_t)std::min<int32_t>((int32_t)matCount - 1, std::max<int32_t>(0, list[i].mat));
    hpar[s].n = newN;
    hpar[s].nFluid = newFluid;
    hpar[s].bondDirty = 1;
    hw.nAct += k;
    update_features();
    hw.hasFriction = hasFriction;
    hw.hasBonds = hasBonds;
    ok = push_scene(s) &&
         cuda_ok(cudaMemcpyAsync(b.world, &hw, sizeof(hw), cudaMemcpyHostToDevice, st), "world") &&
         cuda_ok(cudaStreamSynchronize(st), "spawn");
    if (nOut) *nOut = newN;
    return ok;
  }

  // setWalls (src/engine.js:5262-5305).
  bool set_walls(uint32_t s, bool want, bool* onOut) {
    accFresh = false;
    sortedFresh = false;
    SceneHost& h = sh[s];
    if (!h.loaded) return fail("setWalls before loadScene");
    const uint32_t nB = (uint32_t)h.bmat.size();
    bool cur = h.wallsOn;
    if (nB == 0) { h.wallsOn = want; if (onOut) *onOut = want; return true; }
    if (want == cur) { if (onOut) *onOut = cur; return true; }
    if (!pull_params()) return false;
    if (!want) {
      hw.nAct -= h.n - h.nFluid;
      h.n = h.nFluid;
    } else {
      if (h.nFluid + nB > h.cap) { if (onOut) *onOut = cur; return true; }
      std::vector<int32_t> stw((size_t)nB * 8, 0);
      for (uint32_t bb = 0; bb < nB; ++bb) {
        int32_t* w = &stw[(size_t)bb * 8];
        w[0] = h.bpos[2 * bb];
        w[1] = h.bpos[2 * bb + 1];
        w[4] = (int32_t)h.bmat[bb];
        w[6] = h.hasTemp ? h.btemp[bb] : AMBIENT;
        w[7] = h.hasFuel ? h.bfuel[bb] : row(h.bmat[bb])[M_fuel0];
      }
      size_t off = (size_t)h.slotBase + h.nFluid;
      if (!cuda_ok(cudaMemcpyAsync(b.state + off * 8, stw.data(), stw.size() * 4, cudaMemcpyHostToDevice, st), "walls") ||
          !cuda_ok(cudaMemsetAsync(b.stacc + off, 0, sizeof(int2) * nB, st), "walls"))
        return false;
      h.n = h.nFluid + nB;
      hw.nAct += nB;
    }
    h.wallsOn = want;
    hpar[s].n = h.n;
    bool ok = push_scene(s) &&
              cuda_ok(cudaMemcpyAsync(b.world, &hw, sizeof(hw), cudaMemcpyHostToDevice, st), "world") &&
              cuda_ok(cudaStreamSynchronize(st), "walls");
    if (onOut) *onOut = h.wallsOn;
    return ok;
  }

  bool write_state(uint32_t s, const int32_t* state, const int32_t* scratch, size_t n) {
    accFresh = false;
    sortedFresh = false;
    SceneHost& h = sh[s];
    if (!h.loaded) return fail("write_state before loadScene");
    if (n != h.n) return fail("write_state: n = %zu but the loaded scene has %u", n, h.n);
    size_t off = h.slotBase;
    bool ok = cuda_ok(cudaMemcpyAsync(b.state + off * 8, state, n * 32, cudaMemcpyHostToDevice, st), "state");
    if (scratch) ok = ok && cuda_ok(cudaMemcpyAsync(b.stacc + off, scratch, n * 8, cudaMemcpyHostToDevice, st), "stacc");
    else ok = ok && cuda_ok(cudaMemsetAsync(b.stacc + off, 0, n * 8, st), "stacc");
    return ok && cuda_ok(cudaStreamSynchronize(st), "write_state");
  }

  bool check() {
    uint32_t e[4] = {0, 0, 0, 0};
    cudaMemcpyAsync(e, b.err, 16, cudaMemcpyDeviceToHost, st);
    if (!cuda_ok(cudaStreamSynchronize(st), "checkErrors")) return false;
    if (!cuda_ok(cudaGetLastError(), "checkErrors")) return false;
    if (e[0] & ERR_UNSUPPORTED_ROW)
      return fail("a transition produced a seal-class row (containment is not built); results past it are not "
                  "the reference's");
    if (e[0] & ERR_BOND_PARTNER) return fail("a bond partner slot exceeds the 17-bit bond word");
    if (e[0] & ERR_BARRIER)
      return fail("a grid barrier of the persistent solver loop timed out; results past it are not valid");
    if (e[0] & ERR_STAGE_TIMEOUT)
      return fail("a tile's staged copy did not complete within the bounded wait; results past it are not valid");
    return true;
  }

  // Bond rows written by the host (or a checkpoint) may be non-empty: from
  // here on the digest pass reads every row (work[4] is never cleared).
  void mark_bonds_live() { cudaMemsetAsync(b.work + 4, 0xff, 4, st); }

  // Bond rows of scene s from the host (the write half of the reference's
  // readBond/writeBuffer(bond) pair that replaceWhere and sliceBonds use).
  bool write_bonds(uint32_t s, const uint32_t* in, size_t words) {
    SceneHost& h = sh[s];
    if (!h.loaded) return fail("writeBonds before loadScene");
    if (!in || words < (size_t)h.nFluid * BOND_CAP) return fail("bonds: need %u words", h.nFluid * BOND_CAP);
    accFresh = false;
    cudaMemcpyAsync(b.bond + (size_t)h.slotBase * BOND_CAP, in, (size_t)h.nFluid * BOND_CAP * 4,
                    cudaMemcpyHostToDevice, st);
    mark_bonds_live();
    return cuda_ok(cudaStreamSynchronize(st), "writeBonds");
  }

  // eraseWhere's compaction (src/engine.js:6460-6650) for scene s: keep[i]
  // per fluid slot; survivors keep their order and the boundary block follows
  // them; state and stAcc are permuted, bond contents are renumbered (bonds to
  // erased partners and tombstones dropped), and formation runs on the next
  // substep. Clocks, chain and the impulse queue are untouched.
  bool erase(uint32_t s, const uint8_t* keep, size_t nkeep, uint32_t* removedOut) {
    SceneHost& h = sh[s];
    if (!h.loaded) return fail("eraseWhere before loadScene");
    if (!keep || nkeep != h.nFluid) return fail("eraseWhere: need %u keep flags", h.nFluid);
    accFresh = false;
    sortedFresh = false;
    const uint32_t oldF = h.nFluid, n = h.n, nB = n - oldF;
    std::vector<uint32_t> surv;
    for (uint32_t i = 0; i < oldF; ++i)
      if (keep[i]) surv.push_back(i);
    const uint32_t newF = (uint32_t)surv.size();
    if (removedOut) *removedOut = oldF - newF;
    if (newF == oldF) return true;
    const uint32_t newN = newF + nB;
    if (scene_bodies(s) == 0) {
      if (!erase_device(s, keep, oldF, newF)) return false;
    } else if (!erase_host(s, surv)) {
      return false;
    }
    if (!pull_params()) return false;
    h.n = newN;
    h.nFluid = newF;
    hpar[s].n = newN;
    hpar[s].nFluid = newF;
    hpar[s].bondDirty = 1;
    layoutDirty = true;
    eventsDirty = true;
    return push_scene(s) && cuda_ok(cudaStreamSynchronize(st), "erase");
  }

  // eraseWhere's compaction on the device (a scene without bodies): survivor
  // ranks, state and stAcc moved through scratch, bond rows renumbered into
  // the scene's candidate rows (free until the formation that the erase
  // schedules rewrites them) and copied back.
  char* eraseBuf = nullptr;
  size_t eraseCap = 0;
  bool erase_device(uint32_t s, const uint8_t* keep, uint32_t oldF, uint32_t newF) {
    const SceneHost& h = sh[s];
    const size_t n = h.n, cap = capSlots;
    const size_t offStacc = cap * 32, offO2N = offStacc + cap * 8, offN2O = offO2N + cap * 4, offKeep = offN2O + cap * 4;
    const size_t bytes = offKeep + ((cap + 255) & ~(size_t)255) + 256;
    if (eraseCap < bytes) {
      if (eraseBuf) cudaFree(eraseBuf);
      eraseBuf = dalloc<char>(bytes, err);
      eraseCap = eraseBuf ? bytes : 0;
      if (!eraseBuf) return false;
    }
    int4* tState = reinterpret_cast<int4*>(eraseBuf);
    int2* tStacc = reinterpret_cast<int2*>(eraseBuf + offStacc);
    int32_t* o2n = reinterpret_cast<int32_t*>(eraseBuf + offO2N);
    uint32_t* n2o = reinterpret_cast<uint32_t*>(eraseBuf + offN2O);
    uint8_t* dKeep = reinterpret_cast<uint8_t*>(eraseBuf + offKeep);
    uint32_t* dKept = reinterpret_cast<uint32_t*>(eraseBuf + bytes - 256);
    const size_t base = h.slotBase, newN = newF + (n - oldF);
    uint32_t* bondRows = b.bond + base * BOND_CAP;
    uint32_t* scratchRows = b.bondCand + base * BOND_CAP;
    bool ok = cuda_ok(cudaMemcpyAsync(dKeep, keep, oldF, cudaMemcpyHostToDevice, st), "erase keep");
    if (!ok) return false;
    k_erase_rank<<<1, 1024, 0, st>>>(dKeep, oldF, o2n, dKept);
    k_erase_move<<<grid_for(n), 256, 0, st>>>(b.state + base * 8, b.stacc + base, o2n, (uint32_t)n, oldF, newF,
                                              tState, tStacc, n2o);
    if (oldF) k_erase_bonds<<<grid_for(oldF), 256, 0, st>>>(bondRows, o2n, n2o, oldF, newF, scratchRows);
    ok = cuda_ok(cudaMemcpyAsync(b.state + base * 8, tState, newN * 32, cudaMemcpyDeviceToDevice, st), "erase state") &&
         cuda_ok(cudaMemcpyAsync(b.stacc + base, tStacc, newN * 8, cudaMemcpyDeviceToDevice, st), "erase stAcc");
    if (ok && oldF) {
      ok = cuda_ok(cudaMemcpyAsync(bondRows, scratchRows, (size_t)oldF * BOND_CAP * 4, cudaMemcpyDeviceToDevice, st),
                   "erase bonds") &&
           cuda_ok(cudaMemsetAsync(scratchRows, 0, (size_t)oldF * BOND_CAP * 4, st), "erase cand");
      mark_bonds_live();
    }
    uint32_t kept = 0;
    ok = ok && cuda_ok(cudaMemcpyAsync(&kept, dKept, 4, cudaMemcpyDeviceToHost, st), "erase") &&
         cuda_ok(cudaStreamSynchronize(st), "erase");
    if (!ok) return false;
    if (kept != newF) return fail("erase: the device kept %u particles, the host %u", kept, newF);
    return true;
  }

  // The same compaction on the host, for a scene with bodies (their repair
  // reads the compacted state).
  bool erase_host(uint32_t s, const std::vector<uint32_t>& surv) {
    SceneHost& h = sh[s];
    const uint32_t oldF = h.nFluid, n = h.n, nB = n - oldF, newF = (uint32_t)surv.size();
    std::vector<int32_t> stIn((size_t)n * 8), scIn((size_t)n * 2);
    std::vector<uint32_t> bIn((size_t)oldF * BOND_CAP);
    cudaMemcpyAsync(stIn.data(), b.state + (size_t)h.slotBase * 8, stIn.size() * 4, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(scIn.data(), b.stacc + h.slotBase, scIn.size() * 4, cudaMemcpyDeviceToHost, st);
    if (oldF)
      cudaMemcpyAsync(bIn.data(), b.bond + (size_t)h.slotBase * BOND_CAP, bIn.size() * 4, cudaMemcpyDeviceToHost, st);
    if (!cuda_ok(cudaStreamSynchronize(st), "erase read")) return false;
    const uint32_t newN = newF + nB;
    std::vector<int32_t> stOut((size_t)newN * 8), scOut((size_t)newN * 2);
    auto mv = [&](uint32_t src, uint32_t dst) {
      std::memcpy(&stOut[(size_t)dst * 8], &stIn[(size_t)src * 8], 32);
      std::memcpy(&scOut[(size_t)dst * 2], &scIn[(size_t)src * 2], 8);
    };
    for (uint32_t k = 0; k < newF; ++k) mv(surv[k], k);
    for (uint32_t bb = 0; bb < nB; ++bb) mv(oldF + bb, newF + bb);
    std::vector<int32_t> oldToNew(oldF, -1);
    for (uint32_t k = 0; k < newF; ++k) oldToNew[surv[k]] = (int32_t)k;
    std::vector<uint32_t> bOut((size_t)oldF * BOND_CAP, 0u);  // the full old extent: rows past newF end zero
    for (uint32_t k = 0; k < newF; ++k) {
      uint32_t c = 0;
      for (uint32_t q = 0; q < (uint32_t)BOND_CAP; ++q) {
        const uint32_t w = bIn[(size_t)surv[k] * BOND_CAP + q];
        if (w == 0u) break;
        if (w & BOND_TOMB) continue;
        const uint32_t j = w & BOND_J_MASK;
        const int32_t nj = j < oldF ? oldToNew[j] : -1;
        if (nj < 0) continue;
        bOut[(size_t)k * BOND_CAP + c++] = (w & BOND_L0_MASK) | (uint32_t)nj;
      }
    }
    if (!repair_bodies_after_erase(s, surv, stOut)) return false;
    cudaMemcpyAsync(b.state + (size_t)h.slotBase * 8, stOut.data(), stOut.size() * 4, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(b.stacc + h.slotBase, scOut.data(), scOut.size() * 4, cudaMemcpyHostToDevice, st);
    if (oldF) {
      cudaMemcpyAsync(b.bond + (size_t)h.slotBase * BOND_CAP, bOut.data(), bOut.size() * 4, cudaMemcpyHostToDevice, st);
      mark_bonds_live();
    }
    return cuda_ok(cudaStreamSynchronize(st), "erase write");
  }

  // ---- §20 rigid bodies: host side (src/engine.js:2050-2150, 5452-5811) ----------
  // Device records are in world order (`bodies`); a scene's bodies keep their
  // relative order, and a body's index in the reference's API is its position
  // among its scene's bodies.
  struct BodyHost {
    uint32_t scene = 0, tag = 0, first = 0, last = 0, n = 0;
    bool axis = false, user = false;
  };
  std::vector<BodyHost> bodies;

  static double js_round(double x) {  // Math.round: ties towards +infinity
    const double r = std::floor(x);
    return (x - r >= 0.5) ? r + 1.0 : r;
  }
  // buildCosTable (src/engine.js:2062-2068): Q22 cos over a quarter turn, 1024 steps.
  static void build_cos_table(int32_t* T) {
    for (int k = 0; k <= 1024; ++k)
      T[k] = (int32_t)js_round(std::cos(((double)k * 3.141592653589793) / 2048.0) * 4194304.0);
    T[1024] = 0;
    T[1025] = 0;
  }
  static int64_t idiv_rne64(int64_t a, int64_t n) {  // idivRne (src/engine.js:2074-2080)
    if (n <= 0) return 0;
    const bool neg = a < 0;
    const int64_t x = neg ? -a : a;
    int64_t q = x / n;
    const int64_t r2 = 2 * (x - q * n);
    if (r2 > n || (r2 == n && (q & 1) == 1)) q += 1;
    return neg ? -q : q;
  }
  static double isqrt_js(double x) {  // isqrt64 (src/engine.js:2083-2089), on the same doubles
    if (x <= 0) return 0;
    double r = std::floor(std::sqrt(x));
    while (r > 0 && r * r > x) r -= 1;
    while ((r + 1) * (r + 1) <= x) r += 1;
    return r;
  }
  // rigidShifts (src/engine.js:2106-2128)
  static bool rigid_shifts(const std::vector<int32_t>& ox, const std::vector<int32_t>& oy, int32_t& rMax,
                           int32_t& rsh, int32_t& ish, int32_t& osh) {
    const size_t N = ox.size();
    double rm = 0;
    for (size_t k = 0; k < N; ++k) {
      const double a = std::fabs((double)ox[k]), c = std::fabs((double)oy[k]);
      const double m = isqrt_js(a * a + c * c);
      if (m > rm) rm = m;
    }
    rMax = (int32_t)(int64_t)rm;
    rsh = 0;
    while ((rMax >> rsh) > 2048) ++rsh;
    ish = 0;
    for (;;) {
      double sum = 0;
      for (size_t k = 0; k < N; ++k) {
        const double a = (double)(ox[k] >> ish), c = (double)(oy[k] >> ish);
        sum += a * a + c * c;
      }
      if (sum < 1073741824.0) break;
      if (++ish > 30) return false;
    }
    osh = 0;
    while ((double)N * (double)(rMax >> osh) >= 1073741824.0) ++osh;
    return true;
  }
  // rigidInvInertia (src/engine.js:2135-2150), exact.
  static void rigid_inv_inertia(int32_t s, int32_t rsh, int32_t ish, int32_t& invI, int32_t& iq) {
    invI = 0;
    iq = 0;
    if (s <= 0) return;
    const int32_t bl = 32 - __builtin_clz((uint32_t)s);
    const int32_t iqNat = bl - 1 + 2 * ish - rsh;
    const int32_t q0 = std::min(iqNat, 31);
    const int32_t E = q0 + rsh - 2 * ish;
    if (iqNat < 16 || E < 1 || E > 62) return;
    const unsigned __int128 num = (unsigned __int128)683565276u << E, den = (unsigned __int128)(uint32_t)s;
    unsigned __int128 q = num / den;
    const unsigned __int128 r = num - q * den;
    if (2 * r > den || (2 * r == den && (q & 1))) q += 1;
    if (q > 2147483647u) q = 2147483647u;
    invI = (int32_t)q;
    iq = q0;
  }

  uint32_t scene_bodies(uint32_t s) const {
    uint32_t k = 0;
    for (const BodyHost& bh : bodies) k += bh.scene == s;
    return k;
  }
  int world_body(uint32_t s, uint32_t k) const {  // scene-local index -> record index
    for (size_t i = 0; i < bodies.size(); ++i)
      if (bodies[i].scene == s && k-- == 0) return (int)i;
    return -1;
  }
  bool read_records(std::vector<int32_t>& rec, std::vector<int32_t>& drv) {
    rec.assign(bodies.size() * RG_BODY_WORDS, 0);
    drv.assign(bodies.size() * RG_DRIVER_WORDS, 0);
    if (bodies.empty()) return true;
    return cuda_ok(cudaMemcpyAsync(rec.data(), b.rbody, rec.size() * 4, cudaMemcpyDeviceToHost, st), "bodies") &&
           cuda_ok(cudaMemcpyAsync(drv.data(), b.rdrv, drv.size() * 4, cudaMemcpyDeviceToHost, st), "drivers") &&
           cuda_ok(cudaStreamSynchronize(st), "bodies");
  }
  bool write_records(const std::vector<int32_t>& rec, const std::vector<int32_t>& drv) {
    graphValid = false;
    hw.nBodies = (uint32_t)bodies.size();
    if (bodies.empty()) return true;
    return cuda_ok(cudaMemcpyAsync(b.rbody, rec.data(), rec.size() * 4, cudaMemcpyHostToDevice, st), "bodies") &&
           cuda_ok(cudaMemcpyAsync(b.rdrv, drv.data(), drv.size() * 4, cudaMemcpyHostToDevice, st), "drivers") &&
           cuda_ok(cudaStreamSynchronize(st), "bodies");
  }
  // Replace scene s's bodies by (recS, drvS, descS), keeping every other
  // scene's records as they are on the device.
  bool replace_scene_bodies(uint32_t s, const std::vector<int32_t>& recS, const std::vector<int32_t>& drvS,
                            const std::vector<BodyHost>& descS) {
    std::vector<int32_t> rec, drv;
    if (!read_records(rec, drv)) return false;
    std::vector<int32_t> r2, d2;
    std::vector<BodyHost> b2;
    for (size_t i = 0; i < bodies.size(); ++i) {
      if (bodies[i].scene == s) continue;
      r2.insert(r2.end(), rec.begin() + i * RG_BODY_WORDS, rec.begin() + (i + 1) * RG_BODY_WORDS);
      d2.insert(d2.end(), drv.begin() + i * RG_DRIVER_WORDS, drv.begin() + (i + 1) * RG_DRIVER_WORDS);
      b2.push_back(bodies[i]);
    }
    r2.insert(r2.end(), recS.begin(), recS.end());
    d2.insert(d2.end(), drvS.begin(), drvS.end());
    b2.insert(b2.end(), descS.begin(), descS.end());
    if (b2.size() > (size_t)RG_MAX_BODIES) return fail("more than %d rigid bodies", RG_MAX_BODIES);
    bodies = b2;
    return write_records(r2, d2);
  }
  bool drop_scene_bodies(uint32_t s) {
    if (scene_bodies(s) == 0) return true;
    return replace_scene_bodies(s, {}, {}, {});
  }
  bool read_scene_state(uint32_t s, std::vector<int32_t>& stw) {
    const SceneHost& h = sh[s];
    stw.assign((size_t)h.n * 8, 0);
    if (h.n == 0) return true;
    return cuda_ok(cudaMemcpyAsync(stw.data(), b.state + (size_t)h.slotBase * 8, stw.size() * 4,
                                   cudaMemcpyDeviceToHost, st), "state") &&
           cuda_ok(cudaStreamSynchronize(st), "state");
  }
  bool write_scene_state(uint32_t s, const std::vector<int32_t>& stw, uint32_t lo, uint32_t hi) {
    const SceneHost& h = sh[s];
    if (hi < lo) return true;
    accFresh = false;
    sortedFresh = false;
    return cuda_ok(cudaMemcpyAsync(b.state + ((size_t)h.slotBase + lo) * 8, stw.data() + (size_t)lo * 8,
                                   ((size_t)hi - lo + 1) * 32, cudaMemcpyHostToDevice, st), "state") &&
           cuda_ok(cudaStreamSynchronize(st), "state");
  }
  bool mark_bond_dirty(uint32_t s) {
    if (!pull_params()) return false;
    hpar[s].bondDirty = 1;
    return put_word(s, offsetof(ScenePar, bondDirty), 1u);
  }

  // _writeBodyRecord (src/engine.js:5452-5580): members ascending fluid slots
  // of scene s, `stw` its state words. *idx = the body's index in scene s, or
  // -1 where the reference returns null.
  bool write_body_record(uint32_t s, const std::vector<uint32_t>& members, const std::vector<int32_t>& stw,
                         uint32_t tag, const int32_t* pivot, bool user, int32_t* idx) {
    *idx = -1;
    const size_t N = members.size();
    if (N < 4 || scene_bodies(s) >= (uint32_t)RG_MAX_BODIES || bodies.size() >= (size_t)RG_MAX_BODIES) return true;
    auto W = [&](uint32_t i, int w) { return (int64_t)stw[(size_t)i * 8 + w]; };
    int64_t sx = 0, sy = 0, svx = 0, svy = 0;
    for (uint32_t i : members) { sx += W(i, 0); sy += W(i, 1); svx += W(i, 2); svy += W(i, 3); }
    const bool axis = pivot != nullptr;
    const int32_t cx = axis ? pivot[0] : (int32_t)idiv_rne64(sx, (int64_t)N);
    const int32_t cy = axis ? pivot[1] : (int32_t)idiv_rne64(sy, (int64_t)N);
    const int32_t vx = axis ? 0 : (int32_t)idiv_rne64(svx, (int64_t)N);
    const int32_t vy = axis ? 0 : (int32_t)idiv_rne64(svy, (int64_t)N);
    std::vector<int32_t> ox(N), oy(N);
    for (size_t k = 0; k < N; ++k) {
      ox[k] = (int32_t)(W(members[k], 0) - cx);
      oy[k] = (int32_t)(W(members[k], 1) - cy);
    }
    int32_t rMax, rsh, ish, osh;
    if (!rigid_shifts(ox, oy, rMax, rsh, ish, osh)) return fail("body too large for an i32 inertia sum");
    int64_t sumIs2 = 0, gSum = 0;
    for (size_t k = 0; k < N; ++k) {
      const int64_t a = ox[k] >> ish, c = oy[k] >> ish;
      sumIs2 += a * a + c * c;
      gSum += row((uint32_t)W(members[k], 4))[M_grav];
    }
    int32_t invI, iq;
    rigid_inv_inertia((int32_t)sumIs2, rsh, ish, invI, iq);
    int64_t acc = 0;
    for (size_t k = 0; k < N; ++k)
      acc += (int64_t)(ox[k] >> rsh) * (W(members[k], 3) - vy) - (int64_t)(oy[k] >> rsh) * (W(members[k], 2) - vx);
    int64_t omega = 0;
    if (invI != 0) {
      const __int128 num = (__int128)acc * invI, den = (__int128)1 << iq;
      __int128 q = num / den, r = num - q * den;
      if (r < 0) { q -= 1; r += den; }
      if (2 * r > den || (2 * r == den && (q & 1))) q += 1;
      omega = (int64_t)q;
    }
    const int64_t omegaMax = std::max<int64_t>(
        1, std::min<int64_t>(1073741824, ((int64_t)VMAX * 683565276) / std::max<int64_t>(1, rMax)));
    omega = std::max(-omegaMax, std::min(omegaMax, omega));
    std::vector<int32_t> rec(RG_BODY_WORDS, 0), drv(RG_DRIVER_WORDS, 0);
    rec[RB_LIVE] = 1; rec[RB_TAG] = (int32_t)tag;
    rec[RB_FIRST] = (int32_t)members.front(); rec[RB_LAST] = (int32_t)members.back();
    rec[RB_CX] = cx; rec[RB_CY] = cy; rec[RB_VX] = vx; rec[RB_VY] = vy;
    rec[RB_OMEGA] = (int32_t)omega; rec[RB_N] = (int32_t)N;
    rec[RB_SUMIS2] = (int32_t)sumIs2; rec[RB_GSUM] = (int32_t)(uint32_t)(uint64_t)gSum;
    rec[RB_INVI] = invI; rec[RB_IQ] = iq; rec[RB_RSH] = rsh; rec[RB_ISH] = ish; rec[RB_OSH] = osh;
    rec[RB_OMEGAM] = (int32_t)omegaMax; rec[RB_RMAX] = rMax;
    rec[RB_CQX] = cx; rec[RB_CQY] = cy; rec[RB_AXIS] = axis ? 1 : 0; rec[RB_USER] = user ? 1 : 0;
    rec[RB_SCENE] = (int32_t)s;
    // rest offsets, one copy per contiguous run of member slots
    const uint32_t base = sh[s].slotBase;
    for (size_t k0 = 0; k0 < N;) {
      size_t k1 = k0 + 1;
      while (k1 < N && members[k1] == members[k1 - 1] + 1) ++k1;
      std::vector<int2> win(k1 - k0);
      for (size_t q = k0; q < k1; ++q) win[q - k0] = make_int2(ox[q], oy[q]);
      if (!cuda_ok(cudaMemcpyAsync(b.rest + base + members[k0], win.data(), win.size() * sizeof(int2),
                                   cudaMemcpyHostToDevice, st), "rest") ||
          !cuda_ok(cudaStreamSynchronize(st), "rest"))
        return false;
      k0 = k1;
    }
    const uint32_t at = (uint32_t)bodies.size();
    BodyHost bh;
    bh.scene = s; bh.tag = tag; bh.first = members.front(); bh.last = members.back(); bh.n = (uint32_t)N;
    bh.axis = axis; bh.user = user;
    bodies.push_back(bh);
    *idx = (int32_t)scene_bodies(s) - 1;
    graphValid = false;
    hw.nBodies = (uint32_t)bodies.size();
    return cuda_ok(cudaMemcpyAsync(b.rbody + (size_t)at * RG_BODY_WORDS, rec.data(), RG_BODY_WORDS * 4,
                                   cudaMemcpyHostToDevice, st), "body") &&
           cuda_ok(cudaMemcpyAsync(b.rdrv + (size_t)at * RG_DRIVER_WORDS, drv.data(), RG_DRIVER_WORDS * 4,
                                   cudaMemcpyHostToDevice, st), "driver") &&
           cuda_ok(cudaStreamSynchronize(st), "body");
  }

  // makeRigidBody / makeAxisBody (src/engine.js:5722-5780)
  bool make_rigid_body(uint32_t s, const uint32_t* slots, uint32_t k, const int32_t* pivot, bool user, int32_t* idx) {
    *idx = -1;
    SceneHost& h = sh[s];
    if (!h.loaded) return fail("makeRigidBody before loadScene");
    if (k == 0 || h.nFluid == 0) return true;
    if (!slots) return fail("slots is NULL");
    std::vector<int32_t> stw;
    if (!read_scene_state(s, stw)) return false;
    std::vector<uint32_t> members;
    for (uint32_t q = 0; q < k; ++q) {
      const uint32_t i = slots[q];
      if (i >= h.nFluid) continue;
      if (row((uint32_t)stw[(size_t)i * 8 + 4])[M_solidMode] != SOLID_RIGID) continue;
      if ((uint32_t)stw[(size_t)i * 8 + 5] & (FLAG_RIGID | FLAG_ANCHOR)) continue;
      members.push_back(i);
    }
    std::sort(members.begin(), members.end());
    members.erase(std::unique(members.begin(), members.end()), members.end());
    if (members.size() < 4) return true;
    std::vector<bool> inUse(4096, false);
    for (uint32_t i = 0; i < h.nFluid; ++i) inUse[((uint32_t)stw[(size_t)i * 8 + 5] & WELD_TAG_MASK) >> 8] = true;
    uint32_t seq = 0;
    for (uint32_t g = 0; g <= 4095; ++g) {
      const uint32_t q = next_weld_seq(s);
      if (!inUse[q]) { seq = q; break; }
    }
    if (seq == 0) return fail("§20: no free weld tag for a new body");
    const uint32_t tag = (seq << 8) & WELD_TAG_MASK;
    for (uint32_t i : members) {
      uint32_t& fl = reinterpret_cast<uint32_t&>(stw[(size_t)i * 8 + 5]);
      fl = (fl & ~WELD_TAG_MASK) | tag | FLAG_RIGID;
    }
    if (!write_body_record(s, members, stw, tag, pivot, user, idx)) return false;
    if (*idx < 0) return true;
    return write_scene_state(s, stw, members.front(), members.back()) && mark_bond_dirty(s);
  }
  // The body-record writer the reference's host-side rebuilds call directly
  // (splitDisconnectedBodies, promoteLooseRigidComponents: src/engine.js:
  // 5630-5700, 6313-6430): `members` as given (the caller filtered them), a
  // fresh tag from _nextWeldSeq when tag == 0, FLAG_RIGID and the tag set on
  // them, formation on the next substep.
  bool write_body(uint32_t s, const uint32_t* slots, uint32_t k, uint32_t tag, const int32_t* pivot, bool user,
                  int32_t* idx, uint32_t* tagOut) {
    *idx = -1;
    SceneHost& h = sh[s];
    if (!h.loaded) return fail("writeBodyRecord before loadScene");
    if (k > 0 && !slots) return fail("slots is NULL");
    std::vector<uint32_t> members(slots, slots + k);
    std::sort(members.begin(), members.end());
    members.erase(std::unique(members.begin(), members.end()), members.end());
    if (!members.empty() && members.back() >= h.nFluid) return fail("body member outside the fluid slots");
    const uint32_t t = tag != 0 ? (tag & WELD_TAG_MASK) : ((next_weld_seq(s) << 8) & WELD_TAG_MASK);
    if (tagOut) *tagOut = t;
    if (members.empty()) return true;
    std::vector<int32_t> stw;
    if (!read_scene_state(s, stw)) return false;
    for (uint32_t i : members) {
      uint32_t& fl = reinterpret_cast<uint32_t&>(stw[(size_t)i * 8 + 5]);
      fl = (fl & ~WELD_TAG_MASK) | t | FLAG_RIGID;
    }
    if (!write_body_record(s, members, stw, t, pivot, user, idx)) return false;
    return write_scene_state(s, stw, members.front(), members.back()) && mark_bond_dirty(s);
  }
  // promoteWeldGroup (src/engine.js:5584-5622): the held (or given) tag's
  // rigid-row particles that are neither anchored nor already in a body.
  bool promote_weld_group(uint32_t s, uint32_t tag, const int32_t* pivot, bool user, int32_t* idx) {
    *idx = -1;
    SceneHost& h = sh[s];
    if (!h.loaded) return fail("promoteWeldGroup before loadScene");
    const uint32_t t = (tag == 0 ? h.weldHold : tag) & WELD_TAG_MASK;
    if (t == 0 || h.nFluid == 0) return true;
    std::vector<int32_t> stw;
    if (!read_scene_state(s, stw)) return false;
    std::vector<uint32_t> members;
    for (uint32_t i = 0; i < h.nFluid; ++i) {
      const uint32_t fl = (uint32_t)stw[(size_t)i * 8 + 5];
      if ((fl & WELD_TAG_MASK) != t || (fl & (FLAG_RIGID | FLAG_ANCHOR))) continue;
      if (row((uint32_t)stw[(size_t)i * 8 + 4])[M_solidMode] != SOLID_RIGID) continue;
      members.push_back(i);
    }
    if (!write_body_record(s, members, stw, t, pivot, user, idx)) return false;
    if (*idx < 0) return true;
    for (uint32_t i : members) stw[(size_t)i * 8 + 5] |= (int32_t)FLAG_RIGID;
    return write_scene_state(s, stw, members.front(), members.back()) && mark_bond_dirty(s);
  }
  bool end_weld_group_and_promote(uint32_t s, const int32_t* pivot, bool user, int32_t* idx) {
    *idx = -1;
    uint32_t was = 0;
    if (!end_weld_group(s, &was)) return false;
    if (was == 0) return true;
    return promote_weld_group(s, was, pivot, user, idx);
  }
  // dissolveAllBodies (src/engine.js:5789-5808)
  bool dissolve_all_bodies(uint32_t s, uint32_t* count) {
    if (count) *count = 0;
    if (!sh[s].loaded) return fail("dissolveAllBodies before loadScene");
    if (scene_bodies(s) == 0) return true;
    std::vector<int32_t> stw;
    if (!read_scene_state(s, stw)) return false;
    uint32_t k = 0;
    for (uint32_t i = 0; i < sh[s].nFluid; ++i) {
      int32_t& fl = stw[(size_t)i * 8 + 5];
      if (!((uint32_t)fl & FLAG_RIGID)) continue;
      fl &= ~(int32_t)FLAG_RIGID;
      ++k;
    }
    if (count) *count = k;
    return write_scene_state(s, stw, 0, sh[s].n - 1) && drop_scene_bodies(s);
  }
  bool set_body_user(uint32_t s, uint32_t k, bool on, bool* found) {
    *found = false;
    const int wi = world_body(s, k);
    if (wi < 0) return true;
    bodies[wi].user = on;
    *found = true;
    const int32_t v = on ? 1 : 0;
    return cuda_ok(cudaMemcpyAsync(b.rbody + (size_t)wi * RG_BODY_WORDS + RB_USER, &v, 4, cudaMemcpyHostToDevice, st),
                   "user") &&
           cuda_ok(cudaStreamSynchronize(st), "user");
  }
  // A body's driver sidecar (the words `_serviceBodyConstraints` uploads,
  // src/engine.js:5370-5412): mask of RD_HAS_* bits and the nine values.
  bool set_body_driver(uint32_t s, uint32_t k, int32_t mask, const int32_t* values) {
    const int wi = world_body(s, k);
    if (wi < 0) return fail("body %u is not live", k);
    if (mask < 0 || mask >= 512) return fail("driver mask %d outside 0..511", mask);
    int32_t d[RG_DRIVER_WORDS] = {mask};
    for (int q = 0; q < 9; ++q) d[1 + q] = values ? values[q] : 0;
    return cuda_ok(cudaMemcpyAsync(b.rdrv + (size_t)wi * RG_DRIVER_WORDS, d, sizeof(d), cudaMemcpyHostToDevice, st),
                   "driver") &&
           cuda_ok(cudaStreamSynchronize(st), "driver");
  }
  bool clear_body_drivers(uint32_t s) {
    const int32_t z[RG_DRIVER_WORDS] = {0};
    for (size_t i = 0; i < bodies.size(); ++i)
      if (bodies[i].scene == s &&
          !cuda_ok(cudaMemcpyAsync(b.rdrv + i * RG_DRIVER_WORDS, z, sizeof(z), cudaMemcpyHostToDevice, st), "driver"))
        return false;
    return cuda_ok(cudaStreamSynchronize(st), "driver");
  }
  // dragGrab's rigid branch (src/engine.js:6111-6140)
  bool drag_body(uint32_t s, uint32_t tag, int32_t tx, int32_t ty, int32_t vx, int32_t vy, bool* moved) {
    *moved = false;
    for (size_t i = 0; i < bodies.size(); ++i) {
      if (bodies[i].scene != s || bodies[i].tag != tag) continue;
      if (bodies[i].axis) return true;
      const int32_t cvx = std::max(-VMAX, std::min(VMAX, vx)), cvy = std::max(-VMAX, std::min(VMAX, vy));
      const int64_t ONE = 65536;
      const int32_t w4[4] = {
          (int32_t)std::max<int64_t>(ONE, std::min<int64_t>((int64_t)sh[s].domW - ONE, (int64_t)tx - cvx)),
          (int32_t)std::max<int64_t>(ONE, std::min<int64_t>((int64_t)sh[s].domH - ONE, (int64_t)ty - cvy)), cvx, cvy};
      const int32_t z4[4] = {0, 0, 0, 0};
      *moved = true;
      return cuda_ok(cudaMemcpyAsync(b.rbody + i * RG_BODY_WORDS + RB_CX, w4, 16, cudaMemcpyHostToDevice, st), "drag") &&
             cuda_ok(cudaMemcpyAsync(b.rbody + i * RG_BODY_WORDS + RB_RESX, z4, 16, cudaMemcpyHostToDevice, st), "drag") &&
             cuda_ok(cudaStreamSynchronize(st), "drag");
    }
    return true;
  }
  // readBodies: scene s's records in the reference's layout (word 29 zero).
  bool read_bodies(uint32_t s, int32_t* out, size_t words, uint32_t* count) {
    std::vector<int32_t> rec, drv;
    if (!read_records(rec, drv)) return false;
    const uint32_t nb = scene_bodies(s);
    if (count) *count = nb;
    if (!out) return true;
    if (words < (size_t)nb * RG_BODY_WORDS) return fail("readBodies needs %u words", nb * RG_BODY_WORDS);
    size_t o = 0;
    for (size_t i = 0; i < bodies.size(); ++i) {
      if (bodies[i].scene != s) continue;
      std::memcpy(out + o, rec.data() + i * RG_BODY_WORDS, RG_BODY_WORDS * 4);
      out[o + RB_SCENE] = 0;
      o += RG_BODY_WORDS;
    }
    return true;
  }
  bool read_rest(uint32_t s, int32_t* out, size_t words) {
    const SceneHost& h = sh[s];
    if (!out || words < (size_t)h.n * 2) return fail("readRestOffsets needs n*2 words");
    return h.n == 0 || (cuda_ok(cudaMemcpyAsync(out, b.rest + h.slotBase, (size_t)h.n * 8, cudaMemcpyDeviceToHost, st),
                                "rest") &&
                        cuda_ok(cudaStreamSynchronize(st), "rest"));
  }
  // restoreAuthoringSnapshot's rigid part (src/engine.js:5838-5880).
  bool restore_bodies(uint32_t s, const int32_t* records, uint32_t nb, const int32_t* rest, size_t restWords) {
    if (!sh[s].loaded) return fail("restore before loadScene");
    if (nb > (uint32_t)RG_MAX_BODIES || (nb && !records)) return fail("bad body records");
    if (rest && restWords > (size_t)sh[s].cap * 2) return fail("rest offsets exceed the scene's slots");
    std::vector<int32_t> rec(records, records + (size_t)nb * RG_BODY_WORDS), drv((size_t)nb * RG_DRIVER_WORDS, 0);
    if (rest && restWords &&
        (!cuda_ok(cudaMemcpyAsync(b.rest + sh[s].slotBase, rest, restWords * 4, cudaMemcpyHostToDevice, st), "rest") ||
         !cuda_ok(cudaStreamSynchronize(st), "rest")))
      return false;
    return bodies_from_records(s, rec, drv);
  }
  // Scene s's bodies become the given records (their scene word set to s)
  // and driver sidecars.
  bool bodies_from_records(uint32_t s, std::vector<int32_t> rec, const std::vector<int32_t>& drv) {
    const uint32_t nb = (uint32_t)(rec.size() / RG_BODY_WORDS);
    std::vector<BodyHost> desc(nb);
    for (uint32_t k = 0; k < nb; ++k) {
      int32_t* R = rec.data() + (size_t)k * RG_BODY_WORDS;
      R[RB_SCENE] = (int32_t)s;
      desc[k].scene = s; desc[k].tag = (uint32_t)R[RB_TAG]; desc[k].first = (uint32_t)R[RB_FIRST];
      desc[k].last = (uint32_t)R[RB_LAST]; desc[k].n = (uint32_t)R[RB_N];
      desc[k].axis = R[RB_AXIS] != 0; desc[k].user = R[RB_USER] != 0;
    }
    return replace_scene_bodies(s, rec, drv, desc);
  }
  // eraseWhere's body repair (src/engine.js:6526-6610), on the host copy of
  // the compacted state `stOut` (its flags change here) before it is written.
  bool repair_bodies_after_erase(uint32_t s, const std::vector<uint32_t>& surv, std::vector<int32_t>& stOut) {
    if (scene_bodies(s) == 0) return true;
    const SceneHost& h = sh[s];
    std::vector<int32_t> rec, drv;
    if (!read_records(rec, drv)) return false;
    std::vector<int2> restIn(h.nFluid > 0 ? h.nFluid : 1), restOut(h.cap);
    if (h.nFluid &&
        (!cuda_ok(cudaMemcpyAsync(restIn.data(), b.rest + h.slotBase, (size_t)h.nFluid * 8, cudaMemcpyDeviceToHost, st),
                  "rest") ||
         !cuda_ok(cudaStreamSynchronize(st), "rest")))
      return false;
    const uint32_t newF = (uint32_t)surv.size();
    for (uint32_t k = 0; k < (uint32_t)h.cap; ++k) restOut[k] = make_int2(0, 0);
    for (uint32_t k = 0; k < newF; ++k) restOut[k] = restIn[surv[k]];
    std::vector<int32_t> recS, drvS;
    std::vector<BodyHost> descS;
    for (size_t i = 0; i < bodies.size(); ++i) {
      if (bodies[i].scene != s) continue;
      std::vector<uint32_t> mem;
      for (uint32_t k = 0; k < newF; ++k) {
        const uint32_t fl = (uint32_t)stOut[(size_t)k * 8 + 5];
        if ((fl & FLAG_RIGID) && (fl & WELD_TAG_MASK) == bodies[i].tag) mem.push_back(k);
      }
      if (mem.size() < 4) {
        for (uint32_t k : mem) stOut[(size_t)k * 8 + 5] &= ~(int32_t)FLAG_RIGID;
        continue;
      }
      std::vector<int32_t> r(rec.begin() + i * RG_BODY_WORDS, rec.begin() + (i + 1) * RG_BODY_WORDS);
      const int32_t ish = r[RB_ISH];
      int64_t sumIs2 = 0, gSum = 0;
      for (uint32_t k : mem) {
        const int64_t a = restOut[k].x >> ish, c = restOut[k].y >> ish;
        sumIs2 += a * a + c * c;
        gSum += row((uint32_t)stOut[(size_t)k * 8 + 4])[M_grav];
      }
      int32_t invI, iq;
      rigid_inv_inertia((int32_t)sumIs2, r[RB_RSH], ish, invI, iq);
      r[RB_FIRST] = (int32_t)mem.front(); r[RB_LAST] = (int32_t)mem.back(); r[RB_N] = (int32_t)mem.size();
      r[RB_SUMIS2] = (int32_t)sumIs2; r[RB_GSUM] = (int32_t)(uint32_t)(uint64_t)gSum;
      r[RB_INVI] = invI; r[RB_IQ] = iq;
      recS.insert(recS.end(), r.begin(), r.end());
      drvS.insert(drvS.end(), drv.begin() + i * RG_DRIVER_WORDS, drv.begin() + (i + 1) * RG_DRIVER_WORDS);
      BodyHost d = bodies[i];
      d.first = mem.front(); d.last = mem.back(); d.n = (uint32_t)mem.size();
      descS.push_back(d);
    }
    if (!cuda_ok(cudaMemcpyAsync(b.rest + h.slotBase, restOut.data(), (size_t)h.cap * 8, cudaMemcpyHostToDevice, st),
                 "rest") ||
        !cuda_ok(cudaStreamSynchronize(st), "rest"))
      return false;
    return replace_scene_bodies(s, recS, drvS, descS);
  }

  // ---- material rows at run time: §25 interned rows, §26.C gravity scale ------
  // _internUpload (src/engine.js:5190-5205): one row into the table, rampInv
  // baked from its ramp, grav scaled by the world gravity. `row` may be the
  // next free row (the table grows) or an existing row past the authored ones.
  bool upload_mats(uint32_t lo, uint32_t hi) {
    if (hi <= lo) return true;
    graphValid = false;
    accFresh = false;
    return cuda_ok(cudaMemcpyAsync(const_cast<int32_t*>(b.mats) + (size_t)lo * MAT_WORDS, hmats + (size_t)lo * MAT_WORDS,
                                   sizeof(int32_t) * MAT_WORDS * (hi - lo), cudaMemcpyHostToDevice, st),
                   "mats") &&
           cuda_ok(cudaStreamSynchronize(st), "mats");
  }
  int32_t scaled_grav(int32_t g) const { return (int32_t)idiv_rne64((int64_t)g * gravQ, 65536); }
  bool set_material(uint32_t rowId, const int32_t* w) {
    if (!w) return fail("material words are NULL");
    if (rowId < authoredCount) return fail("row %u is an authored row", rowId);
    if (rowId > matCount || rowId >= (uint32_t)MAT_MAX) return fail("row %u is not the next free row or a minted one", rowId);
    const uint32_t count = std::max(matCount, rowId + 1);
    if (w[M_eps] < 32768) return fail("row %u: eps < 32768", rowId);
    if (w[M_dpMax] <= 0) return fail("row %u: dpMax <= 0", rowId);
    if (w[M_burstP] < 0) return fail("row %u: burstP < 0", rowId);
    if (w[M_sealMode] != 0 && w[M_sealMode] != 1) return fail("row %u: sealMode must be 0 or 1", rowId);
    if ((int64_t)w[M_rampHi] - w[M_rampLo] < 65536) return fail("row %u: ramp narrower than 1 degree", rowId);
    for (int f : {M_meltTo, M_freezeTo, M_boilTo, M_condTo, M_burnTo, M_splitTo, M_corrTo})
      if (w[f] < 0 || (uint32_t)w[f] >= count) return fail("row %u names a product outside the table", rowId);
    int32_t* a = hauth + (size_t)rowId * MAT_WORDS;
    std::memcpy(a, w, sizeof(int32_t) * MAT_WORDS);
    const int64_t span = (int64_t)a[M_rampHi] - a[M_rampLo];
    a[M_rampInv] = span > 0 ? (int32_t)((int64_t)4294967296LL / span) : 0;
    int32_t* d = hmats + (size_t)rowId * MAT_WORDS;
    std::memcpy(d, a, sizeof(int32_t) * MAT_WORDS);
    d[M_grav] = scaled_grav(a[M_grav]);
    matCount = count;
    update_features();
    return upload_mats(rowId, rowId + 1);
  }
  // clearInterned (src/engine.js:5235-5245): drop every row past the authored ones.
  bool clear_materials() {
    for (uint32_t m = authoredCount; m < (uint32_t)MAT_MAX; ++m) {
      std::memset(hauth + (size_t)m * MAT_WORDS, 0, sizeof(int32_t) * MAT_WORDS);
      std::memset(hmats + (size_t)m * MAT_WORDS, 0, sizeof(int32_t) * MAT_WORDS);
    }
    matCount = authoredCount;
    update_features();
    return upload_mats(authoredCount, MAT_MAX);
  }
  // setGravityScale (src/engine.js:4843-4855): q in Q16, clamped to [0, 4].
  bool set_gravity_scale(int32_t q, int32_t* out) {
    const int32_t qq = std::max(0, std::min(4 * 65536, q));
    if (out) *out = qq;
    if (qq == gravQ) return true;
    gravQ = qq;
    for (uint32_t m = 0; m < matCount; ++m)
      hmats[(size_t)m * MAT_WORDS + M_grav] = scaled_grav(hauth[(size_t)m * MAT_WORDS + M_grav]);
    return upload_mats(0, matCount);
  }

  // ---- weld groups (src/engine.js:4570-4680) -----------------------------------
  // _nextWeldSeq: the next 12-bit tag sequence that is neither held open nor
  // worn by one of the scene's bodies.
  bool weld_seq_taken(uint32_t s, uint32_t q) const {
    if (q == sh[s].weldHoldSeq) return true;
    for (const BodyHost& bh : bodies)
      if (bh.scene == s && (bh.tag >> 8) == q) return true;
    return false;
  }
  uint32_t next_weld_seq(uint32_t s) {
    SceneHost& h = sh[s];
    const uint32_t MAXS = 4095;
    uint32_t q = (h.weldSeq % MAXS) + 1;
    for (uint32_t guard = 0; guard <= MAXS && weld_seq_taken(s, q); ++guard) q = (q % MAXS) + 1;
    h.weldSeq = q;
    return q;
  }
  // One ScenePar word, written in stream order without touching the clocks.
  bool put_word(uint32_t s, size_t off, uint32_t v) {
    return cuda_ok(cudaMemcpyAsync(reinterpret_cast<char*>(b.scenes + s) + off, &v, 4, cudaMemcpyHostToDevice, st),
                   "param") &&
           cuda_ok(cudaStreamSynchronize(st), "param");
  }
  bool set_weld_hold(uint32_t s, uint32_t tag) {
    sh[s].weldHold = tag;
    sh[s].weldHoldSeq = tag >> 8;
    hpar[s].weldHold = tag;
    return put_word(s, offsetof(ScenePar, weldHold), tag);
  }
  bool set_fuse(uint32_t s, uint32_t tag) {
    sh[s].fuseTag = tag;
    hpar[s].fuseTag = tag;
    return put_word(s, offsetof(ScenePar, fuseTag), tag);
  }
  bool hold_weld_group(uint32_t s, uint32_t tag, uint32_t* out) {
    if (!sh[s].loaded) return fail("holdWeldGroup before loadScene");
    const uint32_t t = tag & WELD_TAG_MASK;
    if (t == 0) return fail("holdWeldGroup(0): use endWeldGroup() to release");
    if (out) *out = t;
    return set_weld_hold(s, t);
  }
  bool end_weld_group(uint32_t s, uint32_t* was) {
    if (!sh[s].loaded) return fail("endWeldGroup before loadScene");
    if (was) *was = sh[s].weldHold;
    if (sh[s].weldHold == 0) return true;
    if (!set_weld_hold(s, 0)) return false;
    // the formation pass that clears the released tag runs on the next substep
    if (!pull_params()) return false;
    hpar[s].bondDirty = 1;
    return put_word(s, offsetof(ScenePar, bondDirty), 1u);
  }
  bool begin_weld_group(uint32_t s, uint32_t* tag) {
    if (!sh[s].loaded) return fail("beginWeldGroup before loadScene");
    if (sh[s].weldHold != 0 && !end_weld_group(s, nullptr)) return false;
    if (sh[s].fuseTag != 0 && !set_fuse(s, 0)) return false;
    return hold_weld_group(s, (next_weld_seq(s) << 8) & WELD_TAG_MASK, tag);
  }
  bool arm_fuse(uint32_t s, uint32_t* tag) {
    if (!sh[s].loaded) return fail("armFuse before loadScene");
    if (sh[s].weldHold == 0) return fail("armFuse(): no weld group is open");
    if (tag) *tag = sh[s].weldHold;
    return set_fuse(s, sh[s].weldHold);
  }

  // setUserDrive (src/engine.js:4797-4806): clamped to +-USER_A_MAX (32768),
  // read by user-flagged bodies in rigidStep.
  bool set_user_drive(uint32_t s, int32_t ax, int32_t ay, int32_t* out) {
    if (!sh[s].loaded) return fail("setUserDrive before loadScene");
    const int32_t M = 32768;
    const int32_t q[2] = {std::max(-M, std::min(M, ax)), std::max(-M, std::min(M, ay))};
    if (out) { out[0] = q[0]; out[1] = q[1]; }
    if (q[0] == hpar[s].userA[0] && q[1] == hpar[s].userA[1]) return true;
    hpar[s].userA[0] = q[0];
    hpar[s].userA[1] = q[1];
    return put_word(s, offsetof(ScenePar, userA), (uint32_t)q[0]) &&
           put_word(s, offsetof(ScenePar, userA) + 4, (uint32_t)q[1]);
  }

  // setJets (src/engine.js:4740-4770): the first 8 jets, [x, y, r, fx, fy].
  bool set_jets(uint32_t s, const int32_t* q, uint32_t k, uint32_t* nOut) {
    if (!sh[s].loaded) return fail("setJets before loadScene");
    if (k > 0 && !q) return fail("jets is NULL");
    if (k > 8) k = 8;
    if (!pull_params()) return false;
    hpar[s].nJets = k;
    for (uint32_t j = 0; j < 8; ++j)
      for (int w = 0; w < 5; ++w) hpar[s].jet[j][w] = j < k ? q[j * 5 + w] : 0;
    if (nOut) *nOut = k;
    return push_scene(s) && cuda_ok(cudaStreamSynchronize(st), "setJets");
  }

  // Device checkpoint of scene s: [state n*8][stAcc n*2][chain 8][bond rows nFluid*48 when the
  // world has bonding rows], copied on the engine stream.
  // Pool layout of a 2D checkpoint: state (n x 32 B), stAcc (n x 8 B), the
  // chain (32 B), bond rows when the world has bonds, rest offsets (n x 8 B)
  // when the scene has rigid bodies.
  size_t ckpt_bytes(uint32_t s) const {
    const SceneHost& h = sh[s];
    return (size_t)h.n * 40 + 32 + (hasBonds ? (size_t)h.nFluid * BOND_CAP * 4 : 0) +
           (scene_bodies(s) ? (size_t)h.n * 8 : 0);
  }
  bool ckpt_save(uint32_t s, sn_ckpt_pool* pool, uint64_t* handle) {
    SceneHost& h = sh[s];
    if (!h.loaded) return fail("checkpoint of a scene that is not loaded");
    if (pool->device != device) return fail("checkpoint pool is on device %d, the engine on %d", pool->device, device);
    if (layoutDirty && !relayout()) return false;
    if (!pull_params()) return false;
    sn_ckpt_pool::Rec* r = nullptr;
    if (!pool->reserve(ckpt_bytes(s), 2, handle, &r)) return fail("%s", pool->err.c_str());
    char* d = pool->base + r->off;
    const size_t n = h.n;
    bool ok = cuda_ok(cudaMemcpyAsync(d, b.state + (size_t)h.slotBase * 8, n * 32, cudaMemcpyDeviceToDevice, st), "ckpt") &&
              cuda_ok(cudaMemcpyAsync(d + n * 32, b.stacc + h.slotBase, n * 8, cudaMemcpyDeviceToDevice, st), "ckpt") &&
              cuda_ok(cudaMemcpyAsync(d + n * 40, b.chain + (size_t)s * 8, 32, cudaMemcpyDeviceToDevice, st), "ckpt");
    if (ok && hasBonds)
      ok = cuda_ok(cudaMemcpyAsync(d + n * 40 + 32, b.bond + (size_t)h.slotBase * BOND_CAP,
                                   (size_t)h.nFluid * BOND_CAP * 4, cudaMemcpyDeviceToDevice, st), "ckpt");
    r->nBodies = scene_bodies(s);
    r->bodyRec.clear();
    r->bodyDrv.clear();
    if (ok && r->nBodies) {
      const size_t restOff = n * 40 + 32 + (hasBonds ? (size_t)h.nFluid * BOND_CAP * 4 : 0);
      ok = cuda_ok(cudaMemcpyAsync(d + restOff, b.rest + h.slotBase, n * 8, cudaMemcpyDeviceToDevice, st), "ckpt");
      std::vector<int32_t> rec, drv;
      ok = ok && read_records(rec, drv);
      for (size_t i = 0; ok && i < bodies.size(); ++i) {
        if (bodies[i].scene != s) continue;
        r->bodyRec.insert(r->bodyRec.end(), rec.begin() + i * RG_BODY_WORDS, rec.begin() + (i + 1) * RG_BODY_WORDS);
        r->bodyDrv.insert(r->bodyDrv.end(), drv.begin() + i * RG_DRIVER_WORDS,
                          drv.begin() + (i + 1) * RG_DRIVER_WORDS);
      }
    }
    r->n = h.n;
    r->nFluid = h.nFluid;
    r->hasBonds = hasBonds ? 1u : 0u;
    r->substeps = h.substeps;
    r->formClock = hpar[s].formClock;
    r->dirty = hpar[s].bondDirty;
    cudaEventRecord(r->done, st);
    if (!ok) {
      pool->free_rec(*handle);
      return false;
    }
    return true;
  }
  bool ckpt_load(uint32_t s, sn_ckpt_pool* pool, uint64_t handle) {
    accFresh = false;
    sortedFresh = false;
    SceneHost& h = sh[s];
    if (!h.loaded) return fail("checkpoint load into a scene that is not loaded");
    sn_ckpt_pool::Rec* r = pool->find(handle);
    if (!r || r->kind != 2) return fail("no 2D checkpoint %llu in the pool", (unsigned long long)handle);
    if (r->n != h.n || r->nFluid != h.nFluid)
      return fail("checkpoint holds n = %u, n_fluid = %u; the scene has n = %u, n_fluid = %u", r->n, r->nFluid, h.n,
                  h.nFluid);
    if (layoutDirty && !relayout()) return false;
    if (!pull_params()) return false;
    cudaStreamWaitEvent(st, r->done, 0);
    const char* d = pool->base + r->off;
    const size_t n = h.n;
    bool ok = cuda_ok(cudaMemcpyAsync(b.state + (size_t)h.slotBase * 8, d, n * 32, cudaMemcpyDeviceToDevice, st), "load") &&
              cuda_ok(cudaMemcpyAsync(b.stacc + h.slotBase, d + n * 32, n * 8, cudaMemcpyDeviceToDevice, st), "load") &&
              cuda_ok(cudaMemcpyAsync(b.chain + (size_t)s * 8, d + n * 40, 32, cudaMemcpyDeviceToDevice, st), "load");
    uint32_t* bondRows = b.bond + (size_t)h.slotBase * BOND_CAP;
    if (ok && r->hasBonds) {
      ok = cuda_ok(cudaMemcpyAsync(bondRows, d + n * 40 + 32, (size_t)h.nFluid * BOND_CAP * 4,
                                   cudaMemcpyDeviceToDevice, st), "load");
      mark_bonds_live();
    }
    else if (ok)
      ok = cuda_ok(cudaMemsetAsync(bondRows, 0, (size_t)h.nFluid * BOND_CAP * 4, st), "load");
    if (ok && r->nBodies) {
      const size_t restOff = n * 40 + 32 + (r->hasBonds ? (size_t)h.nFluid * BOND_CAP * 4 : 0);
      ok = cuda_ok(cudaMemcpyAsync(b.rest + h.slotBase, d + restOff, n * 8, cudaMemcpyDeviceToDevice, st), "load");
    }
    cudaEventRecord(r->done, st);
    if (!ok) return false;
    // the scene's bodies become the checkpoint's (none if it had none)
    if ((r->nBodies || scene_bodies(s)) && !bodies_from_records(s, r->bodyRec, r->bodyDrv)) return false;
    h.substeps = r->substeps;
    hpar[s].formClock = (uint32_t)r->formClock;
    hpar[s].bondDirty = r->dirty;
    hpar[s].substep = (uint32_t)r->substeps;
    eventsDirty = true;
    return push_scene(s) && cuda_ok(cudaStreamSynchronize(st), "load");
  }

  // Slot allocation for a new scene: first fit over released ranges.
  bool alloc_scene(uint32_t cap, uint32_t* id) {
    uint32_t s = 0;
    while (s < maxScenes && sh[s].used) ++s;
    if (s == maxScenes) return fail("max_scenes reached");
    // find a free slot range [base, base+cap)
    std::vector<std::pair<uint32_t, uint32_t>> usedR;
    for (auto& h : sh)
      if (h.used) usedR.push_back({h.slotBase, h.slotBase + h.cap});
    std::sort(usedR.begin(), usedR.end());
    uint32_t base = 0;
    bool found = false;
    for (auto& r : usedR) {
      if (r.first >= base + cap) { found = true; break; }
      base = std::max(base, r.second);
    }
    if (!found && (uint64_t)base + cap > capSlots) return fail("no room for %u slots", cap);
    sh[s] = SceneHost{};
    sh[s].used = true;
    sh[s].slotBase = base;
    sh[s].cap = cap;
    *id = s;
    layoutDirty = true;
    return true;
  }
};

struct sn_engine {
  World w;
};
struct sn_batch {
  World w;
};

static int rc_of(World& w, bool ok) { return ok ? SN_OK : (w.err.find("cuda") != std::string::npos ? SN_E_CUDA : SN_E_INVALID); }

extern "C" {

int sn_create(const sn_opts* opts, sn_engine** out) {
  if (!out) return SN_E_INVALID;
  *out = nullptr;
  sn_engine* e = new sn_engine();
  if (!e->w.init(opts, 1)) {
    fprintf(stderr, "[suna] create: %s\n", e->w.err.c_str());
    delete e;
    return SN_E_INVALID;
  }
  uint32_t id = 0;
  e->w.alloc_scene(opts->max_particles, &id);
  *out = e;
  return SN_OK;
}
void sn_destroy(sn_engine* e) { delete e; }
const char* sn_last_error(const sn_engine* e) { return e ? e->w.err.c_str() : "null engine"; }
int sn_load_scene(sn_engine* e, const sn_scene* sc) {
  if (!e) return SN_E_INVALID;
  return rc_of(e->w, e->w.load(0, sc));
}
int sn_step(sn_engine* e, uint32_t count, uint64_t* substeps) {
  if (!e) return SN_E_INVALID;
  if (!e->w.sh[0].loaded) { e->w.err = "step() called before loadScene()"; return SN_E_STATE; }
  bool ok = e->w.step(count);
  if (substeps) *substeps = e->w.sh[0].substeps;
  return rc_of(e->w, ok);
}
int sn_digest(sn_engine* e, uint32_t acc[8]) {
  if (!e || !acc) return SN_E_INVALID;
  return rc_of(e->w, e->w.digest(0, acc));
}
int sn_chain(sn_engine* e, uint32_t chain[8]) {
  if (!e || !chain) return SN_E_INVALID;
  return rc_of(e->w, e->w.read_words(e->w.b.chain, chain, 32));
}
int sn_reset_chain(sn_engine* e) {
  if (!e) return SN_E_INVALID;
  return rc_of(e->w, e->w.reset_chain(0) && e->w.cuda_ok(cudaStreamSynchronize(e->w.st), "reset"));
}
int sn_read_state(sn_engine* e, int32_t* out, size_t words) {
  if (!e || !out) return SN_E_INVALID;
  SceneHost& h = e->w.sh[0];
  if (words < (size_t)h.n * 8) { e->w.err = "output buffer too small"; return SN_E_INVALID; }
  return rc_of(e->w, e->w.read_words(e->w.b.state + (size_t)h.slotBase * 8, out, (size_t)h.n * 32));
}
int sn_read_initial_positions(sn_engine* e, int32_t* out, size_t words, size_t* words_out) {
  if (!e || !out) return SN_E_INVALID;
  SceneHost& h = e->w.sh[0];
  if (!h.loaded) { e->w.err = "readInitialPositions before loadScene"; return SN_E_STATE; }
  if (words < (size_t)h.nInit * 2) { e->w.err = "output buffer too small"; return SN_E_INVALID; }
  if (words_out) *words_out = (size_t)h.nInit * 2;
  if (h.nInit == 0) return SN_OK;
  return rc_of(e->w, e->w.read_words(e->w.initPos + h.slotBase, out, (size_t)h.nInit * 8));
}
int sn_read_scratch(sn_engine* e, int32_t* out, size_t words) {
  if (!e || !out) return SN_E_INVALID;
  SceneHost& h = e->w.sh[0];
  if (words < (size_t)h.n * 2) { e->w.err = "output buffer too small"; return SN_E_INVALID; }
  return rc_of(e->w, e->w.read_words(e->w.b.stacc + h.slotBase, out, (size_t)h.n * 8));
}
int sn_write_state(sn_engine* e, const int32_t* state, const int32_t* scratch, size_t n) {
  if (!e || !state) return SN_E_INVALID;
  return rc_of(e->w, e->w.write_state(0, state, scratch, n));
}
int sn_read_bonds(sn_engine* e, uint32_t* out, size_t words) {
  if (!e || !out) return SN_E_INVALID;
  SceneHost& h = e->w.sh[0];
  if (words < (size_t)h.nFluid * BOND_CAP) { e->w.err = "output buffer too small"; return SN_E_INVALID; }
  return rc_of(e->w, e->w.read_words(e->w.b.bond + (size_t)h.slotBase * BOND_CAP, out, (size_t)h.nFluid * BOND_CAP * 4));
}
int sn_read_fields(sn_engine* e, int32_t* rho, uint32_t* nbr_count, size_t n) {
  if (!e) return SN_E_INVALID;
  if (n < (size_t)e->w.sh[0].n) { e->w.err = "output buffer too small"; return SN_E_INVALID; }
  return rc_of(e->w, e->w.read_fields(0, rho, nbr_count));
}
int sn_read_cell_start(sn_engine* e, uint32_t* out, size_t words) {
  if (!e || !out) return SN_E_INVALID;
  World& w = e->w;
  if (!w.sortedFresh || w.layoutDirty) {
    w.err = "no substep has run since the particles last changed";
    return SN_E_INVALID;
  }
  const SceneHost& h = w.sh[0];
  const ScenePar& S = w.hpar[0];
  if (words < (size_t)h.cellTotal + 1) { w.err = "output buffer too small"; return SN_E_INVALID; }
  std::vector<uint32_t> dev((size_t)w.hw.K + 1);
  if (!w.read_words(w.b.cellStart, dev.data(), dev.size() * 4)) return rc_of(w, false);
  // the reference's layout: row-major cells, each cell's first position in a
  // sort by cell index (a prefix sum of the cells' occupancies)
  const uint32_t ts = S.tileShift, T = 1u << ts;
  uint32_t run = 0;
  for (uint32_t cy = 0; cy < h.gridH; ++cy)
    for (uint32_t cx = 0; cx < h.gridW; ++cx) {
      const uint32_t lx = cx & (T - 1u), ly = cy & (T - 1u), c = (lx & 1u) | ((ly & 1u) << 1);
      const uint32_t key = ts == 0u ? S.keyOff[(cx & 1u) | ((cy & 1u) << 1)] + (cy >> 1) * S.nA[(cx & 1u) | ((cy & 1u) << 1)] + (cx >> 1)
                                    : S.keyBase + ((((cy >> ts) * S.tilesX) + (cx >> ts)) << (2u * ts)) +
                                          (c << (2u * ts - 2u)) + (ly >> 1) * (T >> 1) + (lx >> 1);
      out[(size_t)cy * h.gridW + cx] = run;
      run += dev[key + 1] - dev[key];
    }
  out[h.cellTotal] = run;
  return SN_OK;
}
int sn_spawn(sn_engine* e, const sn_particle* list, uint32_t k, uint32_t no_weld, uint32_t* n_out) {
  if (!e || (k && !list)) return SN_E_INVALID;
  return rc_of(e->w, e->w.spawn(0, list, k, (no_weld & SN_SPAWN_NO_WELD) != 0, n_out,
                                (no_weld & SN_SPAWN_OWN_GROUP) != 0));
}
int sn_impulse(sn_engine* e, int32_t cx, int32_t cy, int32_t r, int32_t ix, int32_t iy, uint32_t limit,
               uint32_t* hits) {
  if (!e) return SN_E_INVALID;
  if (!e->w.sh[0].loaded) { e->w.err = "impulse before loadScene"; return SN_E_STATE; }
  return rc_of(e->w, e->w.impulse_now(0, cx, cy, r, ix, iy, limit, hits));
}
int sn_debug_counters(sn_engine* e, uint32_t out[16]) {
  if (!e || !out) return SN_E_INVALID;
  return rc_of(e->w, e->w.read_words(e->w.b.dbg, out, 64));
}
int sn_check_errors(sn_engine* e) {
  if (!e) return SN_E_INVALID;
  if (e->w.check()) return SN_OK;
  return e->w.err.find("cuda") != std::string::npos ? SN_E_CUDA : SN_E_DEVICE;
}
int sn_sync(sn_engine* e) {
  if (!e) return SN_E_INVALID;
  return rc_of(e->w, e->w.cuda_ok(cudaStreamSynchronize(e->w.st), "sync"));
}
int sn_get_info(sn_engine* e, sn_info* out) {
  if (!e || !out) return SN_E_INVALID;
  World& w = e->w;
  if (!w.pull_params()) return SN_E_CUDA;
  SceneHost& h = w.sh[0];
  out->n = h.n;
  out->n_fluid = h.nFluid;
  out->substep_count = h.substeps;
  out->formation_clock = w.hpar[0].formClock;
  out->grid_w = h.gridW;
  out->grid_h = h.gridH;
  out->cell_total = h.cellTotal;
  return SN_OK;
}
int sn_set_formation_clock(sn_engine* e, uint64_t clock, uint32_t dirty) {
  if (!e) return SN_E_INVALID;
  World& w = e->w;
  if (!w.pull_params()) return SN_E_CUDA;
  w.hpar[0].formClock = (uint32_t)clock;
  w.hpar[0].bondDirty = dirty ? 1u : 0u;
  return rc_of(w, w.push_scene(0) && w.cuda_ok(cudaStreamSynchronize(w.st), "clock"));
}
int sn_profile_substep(sn_engine* e, uint32_t reps, float* ms, uint32_t max_phases, uint32_t* n_phases) {
  if (!e || !ms) return SN_E_INVALID;
  if (!e->w.sh[0].loaded) { e->w.err = "profile before loadScene"; return SN_E_STATE; }
  return rc_of(e->w, e->w.profile(reps, ms, max_phases, n_phases));
}
int sn_batch_profile_substep(sn_batch* b, uint32_t reps, float* ms, uint32_t max_phases, uint32_t* n_phases) {
  if (!b || !ms) return SN_E_INVALID;
  return rc_of(b->w, b->w.profile(reps, ms, max_phases, n_phases));
}
int sn_set_walls(sn_engine* e, uint32_t on, uint32_t* walls_on) {
  if (!e) return SN_E_INVALID;
  bool out = false;
  bool ok = e->w.set_walls(0, on != 0, &out);
  if (walls_on) *walls_on = out ? 1u : 0u;
  return rc_of(e->w, ok);
}
int sn_last_timing(sn_engine* e, float* ms, uint64_t* launches) {
  if (!e) return SN_E_INVALID;
  if (ms && !e->w.timing(ms)) return SN_E_CUDA;
  if (launches) *launches = e->w.lastLaunches;
  return SN_OK;
}

// ---- batch ------------------------------------------------------------------
int sn_batch_create(const sn_opts* opts, uint32_t max_scenes, sn_batch** out) {
  if (!out || max_scenes == 0) return SN_E_INVALID;
  *out = nullptr;
  sn_batch* b = new sn_batch();
  if (!b->w.init(opts, max_scenes)) {
    fprintf(stderr, "[suna] batch create: %s\n", b->w.err.c_str());
    delete b;
    return SN_E_INVALID;
  }
  *out = b;
  return SN_OK;
}
void sn_batch_destroy(sn_batch* b) { delete b; }
const char* sn_batch_last_error(const sn_batch* b) { return b ? b->w.err.c_str() : "null batch"; }
int sn_batch_add_scene(sn_batch* b, const sn_scene* sc, uint32_t capacity, uint32_t* id) {
  if (!b || !sc || !id) return SN_E_INVALID;
  World& w = b->w;
  uint32_t cap = std::max(capacity, sc->n);
  uint32_t s = 0;
  if (!w.alloc_scene(cap, &s)) return SN_E_CAPACITY;
  if (!w.load(s, sc)) {
    w.sh[s].used = false;
    w.layoutDirty = true;
    return rc_of(w, false);
  }
  *id = s;
  return SN_OK;
}
int sn_batch_remove_scene(sn_batch* b, uint32_t id) {
  if (!b || id >= b->w.maxScenes || !b->w.sh[id].used) return SN_E_INVALID;
  World& w = b->w;
  if (!w.drop_scene_bodies(id)) return rc_of(w, false);
  w.sh[id] = SceneHost{};
  w.hpar[id] = ScenePar{};
  w.layoutDirty = true;
  w.eventsDirty = true;
  return rc_of(w, w.relayout());
}
int sn_batch_step(sn_batch* b, uint32_t count) {
  if (!b) return SN_E_INVALID;
  return rc_of(b->w, b->w.step(count));
}
int sn_batch_schedule_impulse(sn_batch* b, uint32_t id, uint64_t at, int32_t cx, int32_t cy, int32_t r, int32_t ix,
                              int32_t iy, uint32_t limit) {
  if (!b || id >= b->w.maxScenes || !b->w.sh[id].loaded) return SN_E_INVALID;
  SceneHost& h = b->w.sh[id];
  if (at < h.substeps) { b->w.err = "impulse scheduled in the past"; return SN_E_INVALID; }
  if (!h.events.empty() && at < h.events.back().at) { b->w.err = "impulses must be queued in substep order"; return SN_E_INVALID; }
  if (at > 0xffffffffull) return SN_E_INVALID;
  h.events.push_back(ImpulseEv{(uint32_t)at, cx, cy, r, ix, iy, limit, 0});
  b->w.eventsDirty = true;
  return SN_OK;
}
int sn_batch_digest(sn_batch* b, uint32_t id, uint32_t acc[8]) {
  if (!b || !acc || id >= b->w.maxScenes || !b->w.sh[id].loaded) return SN_E_INVALID;
  return rc_of(b->w, b->w.digest(id, acc));
}
int sn_batch_chain(sn_batch* b, uint32_t id, uint32_t chain[8]) {
  if (!b || !chain || id >= b->w.maxScenes || !b->w.sh[id].loaded) return SN_E_INVALID;
  return rc_of(b->w, b->w.read_words(b->w.b.chain + id * 8, chain, 32));
}
int sn_batch_read_state(sn_batch* b, uint32_t id, int32_t* out, size_t words) {
  if (!b || !out || id >= b->w.maxScenes || !b->w.sh[id].loaded) return SN_E_INVALID;
  SceneHost& h = b->w.sh[id];
  if (words < (size_t)h.n * 8) return SN_E_INVALID;
  return rc_of(b->w, b->w.read_words(b->w.b.state + (size_t)h.slotBase * 8, out, (size_t)h.n * 32));
}
int sn_batch_read_scratch(sn_batch* b, uint32_t id, int32_t* out, size_t words) {
  if (!b || !out || id >= b->w.maxScenes || !b->w.sh[id].loaded) return SN_E_INVALID;
  SceneHost& h = b->w.sh[id];
  if (words < (size_t)h.n * 2) return SN_E_INVALID;
  return rc_of(b->w, b->w.read_words(b->w.b.stacc + h.slotBase, out, (size_t)h.n * 8));
}
int sn_batch_write_state(sn_batch* b, uint32_t id, const int32_t* state, const int32_t* scratch, size_t n,
                         uint64_t substep_count, uint64_t formation_clock, uint32_t dirty) {
  if (!b || !state || id >= b->w.maxScenes || !b->w.sh[id].loaded) return SN_E_INVALID;
  World& w = b->w;
  if (!w.write_state(id, state, scratch, n)) return rc_of(w, false);
  if (!w.pull_params()) return SN_E_CUDA;
  w.sh[id].substeps = substep_count;
  w.hpar[id].formClock = (uint32_t)formation_clock;
  w.hpar[id].bondDirty = dirty ? 1u : 0u;
  w.hpar[id].substep = (uint32_t)substep_count;
  w.eventsDirty = true;
  return rc_of(w, w.push_scene(id) && w.cuda_ok(cudaStreamSynchronize(w.st), "write"));
}
int sn_begin_weld_group(sn_engine* e, uint32_t* tag) {
  if (!e) return SN_E_INVALID;
  return rc_of(e->w, e->w.begin_weld_group(0, tag));
}
int sn_hold_weld_group(sn_engine* e, uint32_t tag) {
  if (!e) return SN_E_INVALID;
  return rc_of(e->w, e->w.hold_weld_group(0, tag, nullptr));
}
int sn_end_weld_group(sn_engine* e, uint32_t* was) {
  if (!e) return SN_E_INVALID;
  return rc_of(e->w, e->w.end_weld_group(0, was));
}
int sn_arm_fuse(sn_engine* e, uint32_t* tag) {
  if (!e) return SN_E_INVALID;
  return rc_of(e->w, e->w.arm_fuse(0, tag));
}
int sn_weld_state(sn_engine* e, uint32_t out[4]) {
  if (!e || !out) return SN_E_INVALID;
  const SceneHost& h = e->w.sh[0];
  out[0] = h.weldHold;
  out[1] = h.fuseTag;
  out[2] = h.lastWeldTag;
  out[3] = h.weldSeq;
  return SN_OK;
}
int sn_write_bonds(sn_engine* e, const uint32_t* bonds, size_t words) {
  if (!e) return SN_E_INVALID;
  return rc_of(e->w, e->w.write_bonds(0, bonds, words));
}
int sn_batch_write_bonds(sn_batch* b, uint32_t id, const uint32_t* bonds, size_t words) {
  if (!b || id >= b->w.maxScenes) return SN_E_INVALID;
  return rc_of(b->w, b->w.write_bonds(id, bonds, words));
}
int sn_erase(sn_engine* e, const uint8_t* keep, size_t n, uint32_t* removed) {
  if (!e) return SN_E_INVALID;
  return rc_of(e->w, e->w.erase(0, keep, n, removed));
}
int sn_batch_erase(sn_batch* b, uint32_t id, const uint8_t* keep, size_t n, uint32_t* removed) {
  if (!b || id >= b->w.maxScenes) return SN_E_INVALID;
  return rc_of(b->w, b->w.erase(id, keep, n, removed));
}
int sn_set_jets(sn_engine* e, const int32_t* jets, uint32_t k, uint32_t* n_out) {
  if (!e) return SN_E_INVALID;
  return rc_of(e->w, e->w.set_jets(0, jets, k, n_out));
}
int sn_batch_set_jets(sn_batch* b, uint32_t id, const int32_t* jets, uint32_t k, uint32_t* n_out) {
  if (!b || id >= b->w.maxScenes) return SN_E_INVALID;
  return rc_of(b->w, b->w.set_jets(id, jets, k, n_out));
}
int sn_set_user_drive(sn_engine* e, int32_t ax, int32_t ay, int32_t out[2]) {
  if (!e) return SN_E_INVALID;
  return rc_of(e->w, e->w.set_user_drive(0, ax, ay, out));
}
int sn_autotune(sn_engine* e, uint32_t reps, uint32_t* substeps_run) {
  if (!e) return SN_E_INVALID;
  return rc_of(e->w, e->w.autotune(reps, substeps_run));
}
int sn_batch_autotune(sn_batch* b, uint32_t reps, uint32_t* substeps_run) {
  if (!b) return SN_E_INVALID;
  return rc_of(b->w, b->w.autotune(reps, substeps_run));
}
int sn_autotune_layout(sn_engine* e, uint32_t reps, uint32_t* substeps_run, uint32_t* layout, float* ms_per_substep) {
  if (!e) return SN_E_INVALID;
  return rc_of(e->w, e->w.autotune_layout(reps, substeps_run, layout, ms_per_substep));
}
int sn_batch_autotune_layout(sn_batch* b, uint32_t reps, uint32_t* substeps_run, uint32_t* layout,
                             float* ms_per_substep) {
  if (!b) return SN_E_INVALID;
  return rc_of(b->w, b->w.autotune_layout(reps, substeps_run, layout, ms_per_substep));
}
int sn_set_tile_shape(sn_engine* e, uint32_t shift) {
  if (!e || shift < TILE_SHIFT_MIN || shift > TILE_SHIFT_MAX) return SN_E_INVALID;
  e->w.tileShiftPinned = shift;
  e->w.layoutDirty = true;
  return SN_OK;
}
int sn_batch_set_tile_shape(sn_batch* b, uint32_t shift) {
  if (!b || shift < TILE_SHIFT_MIN || shift > TILE_SHIFT_MAX) return SN_E_INVALID;
  b->w.tileShiftPinned = shift;
  b->w.layoutDirty = true;
  return SN_OK;
}
int sn_set_staged(sn_engine* e, uint32_t on) {
  if (!e) return SN_E_INVALID;
  e->w.staged = on != 0;
  e->w.layoutDirty = true;
  return SN_OK;
}
int sn_batch_set_staged(sn_batch* b, uint32_t on) {
  if (!b) return SN_E_INVALID;
  b->w.staged = on != 0;
  b->w.layoutDirty = true;
  return SN_OK;
}
int sn_set_persistent(sn_engine* e, uint32_t on) {
  if (!e) return SN_E_INVALID;
  e->w.persistent = on != 0;
  e->w.graphValid = false;
  return SN_OK;
}
int sn_batch_set_persistent(sn_batch* b, uint32_t on) {
  if (!b) return SN_E_INVALID;
  b->w.persistent = on != 0;
  b->w.graphValid = false;
  return SN_OK;
}
int sn_lanes(sn_engine* e, uint32_t out[5]) {
  if (!e || !out) return SN_E_INVALID;
  const auto& c = e->w.lanesCfg;
  out[0] = c.a; out[1] = c.c; out[2] = c.p1; out[3] = c.p2; out[4] = c.n;
  return SN_OK;
}
int sn_set_lanes(sn_engine* e, const uint32_t lanes[5]) {
  if (!e) return SN_E_INVALID;
  return rc_of(e->w, e->w.set_lanes(lanes));
}
int sn_batch_set_lanes(sn_batch* b, const uint32_t lanes[5]) {
  if (!b) return SN_E_INVALID;
  return rc_of(b->w, b->w.set_lanes(lanes));
}
int sn_batch_lanes(sn_batch* b, uint32_t out[5]) {
  if (!b || !out) return SN_E_INVALID;
  const auto& c = b->w.lanesCfg;
  out[0] = c.a; out[1] = c.c; out[2] = c.p1; out[3] = c.p2; out[4] = c.n;
  return SN_OK;
}
int sn_ckpt_pool_create(size_t bytes, int32_t device, sn_ckpt_pool** out) {
  if (!out || bytes == 0) return SN_E_INVALID;
  *out = nullptr;
  if (cudaSetDevice(device) != cudaSuccess) return SN_E_CUDA;
  sn_ckpt_pool* p = new sn_ckpt_pool();
  p->device = device;
  p->cap = sn_ckpt_pool::round_up(bytes);
  if (cudaMalloc(&p->base, p->cap) != cudaSuccess) {
    fprintf(stderr, "[suna] checkpoint pool: cudaMalloc of %zu bytes failed\n", p->cap);
    p->base = nullptr;
    delete p;
    return SN_E_CAPACITY;
  }
  p->freeList[0] = p->cap;
  *out = p;
  return SN_OK;
}
void sn_ckpt_pool_destroy(sn_ckpt_pool* p) { delete p; }
const char* sn_ckpt_pool_last_error(const sn_ckpt_pool* p) { return p ? p->err.c_str() : "null pool"; }
int sn_ckpt_pool_usage(const sn_ckpt_pool* p, size_t* used, size_t* capacity) {
  if (!p) return SN_E_INVALID;
  if (used) *used = p->used;
  if (capacity) *capacity = p->cap;
  return SN_OK;
}
int sn_ckpt_free(sn_ckpt_pool* p, uint64_t handle) {
  if (!p) return SN_E_INVALID;
  return p->free_rec(handle) ? SN_OK : SN_E_INVALID;
}
int sn_ckpt_bytes(sn_engine* e, size_t* bytes) {
  if (!e || !bytes || !e->w.sh[0].loaded) return SN_E_INVALID;
  *bytes = e->w.ckpt_bytes(0);
  return SN_OK;
}
int sn_ckpt_save(sn_engine* e, sn_ckpt_pool* p, uint64_t* handle) {
  if (!e || !p || !handle) return SN_E_INVALID;
  if (e->w.ckpt_save(0, p, handle)) return SN_OK;
  return e->w.err.rfind("checkpoint pool full", 0) == 0 ? SN_E_CAPACITY : rc_of(e->w, false);
}
int sn_ckpt_load(sn_engine* e, sn_ckpt_pool* p, uint64_t handle) {
  if (!e || !p) return SN_E_INVALID;
  return rc_of(e->w, e->w.ckpt_load(0, p, handle));
}
int sn_batch_ckpt_bytes(sn_batch* b, uint32_t id, size_t* bytes) {
  if (!b || !bytes || id >= b->w.maxScenes || !b->w.sh[id].loaded) return SN_E_INVALID;
  *bytes = b->w.ckpt_bytes(id);
  return SN_OK;
}
int sn_batch_ckpt_save(sn_batch* b, uint32_t id, sn_ckpt_pool* p, uint64_t* handle) {
  if (!b || !p || !handle || id >= b->w.maxScenes) return SN_E_INVALID;
  if (b->w.ckpt_save(id, p, handle)) return SN_OK;
  return b->w.err.rfind("checkpoint pool full", 0) == 0 ? SN_E_CAPACITY : rc_of(b->w, false);
}
int sn_batch_ckpt_load(sn_batch* b, uint32_t id, sn_ckpt_pool* p, uint64_t handle) {
  if (!b || !p || id >= b->w.maxScenes) return SN_E_INVALID;
  return rc_of(b->w, b->w.ckpt_load(id, p, handle));
}
int sn_batch_get_info(sn_batch* b, uint32_t id, sn_info* out) {
  if (!b || !out || id >= b->w.maxScenes || !b->w.sh[id].loaded) return SN_E_INVALID;
  World& w = b->w;
  if (!w.pull_params()) return SN_E_CUDA;
  SceneHost& h = w.sh[id];
  out->n = h.n;
  out->n_fluid = h.nFluid;
  out->substep_count = h.substeps;
  out->formation_clock = w.hpar[id].formClock;
  out->grid_w = h.gridW;
  out->grid_h = h.gridH;
  out->cell_total = h.cellTotal;
  return SN_OK;
}
int sn_batch_check_errors(sn_batch* b) {
  if (!b) return SN_E_INVALID;
  return b->w.check() ? SN_OK : SN_E_DEVICE;
}
int sn_batch_sync(sn_batch* b) {
  if (!b) return SN_E_INVALID;
  return rc_of(b->w, b->w.cuda_ok(cudaStreamSynchronize(b->w.st), "sync"));
}
int sn_batch_last_timing(sn_batch* b, float* ms, uint64_t* launches) {
  if (!b) return SN_E_INVALID;
  if (ms && !b->w.timing(ms)) return SN_E_CUDA;
  if (launches) *launches = b->w.lastLaunches;
  return SN_OK;
}


// ---- §20 rigid bodies (src/engine.js:5452-5811) -------------------------------
int sn_make_rigid_body(sn_engine* e, const uint32_t* slots, uint32_t k, const int32_t* pivot, uint32_t user,
                       int32_t* index) {
  if (!e || !index) return SN_E_INVALID;
  return rc_of(e->w, e->w.make_rigid_body(0, slots, k, pivot, user != 0, index));
}
int sn_promote_weld_group(sn_engine* e, uint32_t tag, const int32_t* pivot, uint32_t user, int32_t* index) {
  if (!e || !index) return SN_E_INVALID;
  return rc_of(e->w, e->w.promote_weld_group(0, tag, pivot, user != 0, index));
}
int sn_end_weld_group_and_promote(sn_engine* e, const int32_t* pivot, uint32_t user, int32_t* index) {
  if (!e || !index) return SN_E_INVALID;
  return rc_of(e->w, e->w.end_weld_group_and_promote(0, pivot, user != 0, index));
}
int sn_dissolve_all_bodies(sn_engine* e, uint32_t* count) {
  if (!e) return SN_E_INVALID;
  return rc_of(e->w, e->w.dissolve_all_bodies(0, count));
}
int sn_read_bodies(sn_engine* e, int32_t* out, size_t words, uint32_t* count) {
  if (!e) return SN_E_INVALID;
  return rc_of(e->w, e->w.read_bodies(0, out, words, count));
}
int sn_read_rest_offsets(sn_engine* e, int32_t* out, size_t words) {
  if (!e) return SN_E_INVALID;
  return rc_of(e->w, e->w.read_rest(0, out, words));
}
int sn_set_body_user(sn_engine* e, uint32_t index, uint32_t on, uint32_t* found) {
  if (!e) return SN_E_INVALID;
  bool f = false;
  const bool ok = e->w.set_body_user(0, index, on != 0, &f);
  if (found) *found = f ? 1u : 0u;
  return rc_of(e->w, ok);
}
int sn_set_body_driver(sn_engine* e, uint32_t index, int32_t mask, const int32_t values[9]) {
  if (!e) return SN_E_INVALID;
  return rc_of(e->w, e->w.set_body_driver(0, index, mask, values));
}
int sn_clear_body_drivers(sn_engine* e) {
  if (!e) return SN_E_INVALID;
  return rc_of(e->w, e->w.clear_body_drivers(0));
}
int sn_drag_body(sn_engine* e, uint32_t tag, int32_t x, int32_t y, int32_t vx, int32_t vy, uint32_t* moved) {
  if (!e) return SN_E_INVALID;
  bool m = false;
  const bool ok = e->w.drag_body(0, tag, x, y, vx, vy, &m);
  if (moved) *moved = m ? 1u : 0u;
  return rc_of(e->w, ok);
}
int sn_write_body(sn_engine* e, const uint32_t* members, uint32_t k, uint32_t tag, const int32_t* pivot, uint32_t user,
                  int32_t* index, uint32_t* tag_out) {
  if (!e || !index) return SN_E_INVALID;
  return rc_of(e->w, e->w.write_body(0, members, k, tag, pivot, user != 0, index, tag_out));
}
// The same body calls on one scene of a batch (bodies belong to their scene;
// removing the scene drops them).
#define SN_BATCH_SCENE(b, id) \
  if (!(b) || (id) >= (b)->w.maxScenes) return SN_E_INVALID
int sn_batch_make_rigid_body(sn_batch* b, uint32_t id, const uint32_t* slots, uint32_t k, const int32_t* pivot,
                             uint32_t user, int32_t* index) {
  SN_BATCH_SCENE(b, id);
  if (!index) return SN_E_INVALID;
  return rc_of(b->w, b->w.make_rigid_body(id, slots, k, pivot, user != 0, index));
}
int sn_batch_promote_weld_group(sn_batch* b, uint32_t id, uint32_t tag, const int32_t* pivot, uint32_t user,
                                int32_t* index) {
  SN_BATCH_SCENE(b, id);
  if (!index) return SN_E_INVALID;
  return rc_of(b->w, b->w.promote_weld_group(id, tag, pivot, user != 0, index));
}
int sn_batch_dissolve_all_bodies(sn_batch* b, uint32_t id, uint32_t* count) {
  SN_BATCH_SCENE(b, id);
  return rc_of(b->w, b->w.dissolve_all_bodies(id, count));
}
int sn_batch_read_bodies(sn_batch* b, uint32_t id, int32_t* out, size_t words, uint32_t* count) {
  SN_BATCH_SCENE(b, id);
  return rc_of(b->w, b->w.read_bodies(id, out, words, count));
}
int sn_batch_read_rest_offsets(sn_batch* b, uint32_t id, int32_t* out, size_t words) {
  SN_BATCH_SCENE(b, id);
  return rc_of(b->w, b->w.read_rest(id, out, words));
}
int sn_batch_set_body_user(sn_batch* b, uint32_t id, uint32_t index, uint32_t on, uint32_t* found) {
  SN_BATCH_SCENE(b, id);
  bool f = false;
  const bool ok = b->w.set_body_user(id, index, on != 0, &f);
  if (found) *found = f ? 1u : 0u;
  return rc_of(b->w, ok);
}
int sn_batch_set_body_driver(sn_batch* b, uint32_t id, uint32_t index, int32_t mask, const int32_t values[9]) {
  SN_BATCH_SCENE(b, id);
  return rc_of(b->w, b->w.set_body_driver(id, index, mask, values));
}
int sn_batch_clear_body_drivers(sn_batch* b, uint32_t id) {
  SN_BATCH_SCENE(b, id);
  return rc_of(b->w, b->w.clear_body_drivers(id));
}
int sn_batch_drag_body(sn_batch* b, uint32_t id, uint32_t tag, int32_t x, int32_t y, int32_t vx, int32_t vy,
                       uint32_t* moved) {
  SN_BATCH_SCENE(b, id);
  bool m = false;
  const bool ok = b->w.drag_body(id, tag, x, y, vx, vy, &m);
  if (moved) *moved = m ? 1u : 0u;
  return rc_of(b->w, ok);
}
#undef SN_BATCH_SCENE
int sn_set_material(sn_engine* e, uint32_t row, const int32_t words[48], uint32_t* mat_count) {
  if (!e) return SN_E_INVALID;
  const bool ok = e->w.set_material(row, words);
  if (mat_count) *mat_count = e->w.matCount;
  return rc_of(e->w, ok);
}
int sn_clear_materials(sn_engine* e) {
  if (!e) return SN_E_INVALID;
  return rc_of(e->w, e->w.clear_materials());
}
int sn_set_gravity_scale(sn_engine* e, int32_t q, int32_t* out) {
  if (!e) return SN_E_INVALID;
  return rc_of(e->w, e->w.set_gravity_scale(q, out));
}
int sn_batch_set_material(sn_batch* b, uint32_t row, const int32_t words[48], uint32_t* mat_count) {
  if (!b) return SN_E_INVALID;
  const bool ok = b->w.set_material(row, words);
  if (mat_count) *mat_count = b->w.matCount;
  return rc_of(b->w, ok);
}
int sn_restore_bodies(sn_engine* e, const int32_t* records, uint32_t count, const int32_t* rest, size_t rest_words) {
  if (!e) return SN_E_INVALID;
  return rc_of(e->w, e->w.restore_bodies(0, records, count, rest, rest_words));
}

}  // extern "C"
