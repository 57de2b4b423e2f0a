// Host side of the 3D engine: device buffers, the per-substep launch sequence
// under a CUDA graph, and the sn3_* C ABI declared in include/suna.h.
//
// One sn3_engine holds one or more independent 3D scenes in one set of device
// buffers and advances all of them with one launch sequence per substep; the
// single-scene drop-in for the reference's 3D page (class App in 3d/app.js:
// reset, runSubsteps, spawn, setBallRadius, chain) is scene 0.
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/suna.h"
#include "ckptpool.h"
#include "radix.cuh"
#include "sim3d.cuh"

using namespace sn::d3;
namespace radix = sn::radix;

namespace {

// Scene upload (pos 3n, vel 3n, mat n as uploaded): res[0] = the first
// particle whose material is outside the table.
__global__ void __launch_bounds__(256) k3_load_check(const int32_t* __restrict__ raw, uint32_t n, uint32_t matCount,
                                                     uint32_t* __restrict__ res) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    if ((uint32_t)raw[6 * (size_t)n + i] >= matCount) atomicMin(res, i);
}
// ... and its packing into state words {p.xyz, mat, v.xyz, 0}.
__global__ void __launch_bounds__(256) k3_load_pack(const int32_t* __restrict__ raw, uint32_t n, uint32_t hasVel,
                                                    int32_t* __restrict__ state) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int32_t* pp = raw + 3 * (size_t)i;
    const int32_t* vv = raw + 3 * (size_t)n + 3 * (size_t)i;
    int4* w4 = reinterpret_cast<int4*>(state + (size_t)i * 8);
    w4[0] = make_int4(pp[0], pp[1], pp[2], raw[6 * (size_t)n + i]);
    w4[1] = hasVel ? make_int4(vv[0], vv[1], vv[2], 0) : make_int4(0, 0, 0, 0);
  }
}
// Bond rows as uploaded: res[0] = the first malformed row (an entry after the
// row's end, a rest length on an empty entry, a partner outside the scene or
// itself, a rest length outside [BOND3_L0_MIN, BOND3_L0_MAX]); res[1] != 0 when
// any row holds an entry.
__global__ void __launch_bounds__(256) k3_bonds_check(const uint32_t* __restrict__ rows, uint32_t n,
                                                      uint32_t* __restrict__ res) {
  bool anyRow = false;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t* r = rows + (size_t)i * BOND3_WORDS;
    bool ended = false, bad = false;
    for (uint32_t e = 0; e < BOND3_CAP; ++e) {
      const uint32_t w = r[2 * e], L0 = r[2 * e + 1];
      if (w == 0u) {
        ended = true;
        bad |= L0 != 0u;
        continue;
      }
      const uint32_t j = (w & BOND3_J) - 1u;
      bad |= ended || j >= n || j == i || (int32_t)L0 < BOND3_L0_MIN || (int32_t)L0 > BOND3_L0_MAX;
      anyRow = true;
    }
    if (bad) atomicMin(res, i);
  }
  if (__any_sync(0xffffffffu, anyRow) && (threadIdx.x & 31u) == 0u) atomicOr(res + 1, 1u);
}
// bflag[i] = 1 when row i holds an entry.
__global__ void __launch_bounds__(256) k3_bond_flags(const uint32_t* __restrict__ rows, uint32_t n,
                                                     uint32_t* __restrict__ flag) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    flag[i] = rows[(size_t)i * BOND3_WORDS] != 0u ? 1u : 0u;
}

template <typename T>
T* dalloc3(size_t count, std::string& err) {
  if (count == 0) count = 1;
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, count * sizeof(T));
  if (e != cudaSuccess) {
    if (err.empty()) err = std::string("cudaMalloc: ") + cudaGetErrorString(e);
    return nullptr;
  }
  // The zeroing runs on the legacy default stream, which does not order with
  // the engine's non-blocking stream: finish it before anything is queued there.
  cudaMemset(p, 0, count * sizeof(T));
  cudaDeviceSynchronize();
  return static_cast<T*>(p);
}

// JavaScript's Math.round: the nearest integer, ties toward +infinity.
double js_round(double x) {
  double f = std::floor(x);
  return (x - f >= 0.5) ? f + 1.0 : f;
}

constexpr uint32_t MAT3_MAX = 256;
constexpr int32_t ONE = 65536;

struct Scene3Host {
  bool used = false, loaded = false;
  uint32_t slotBase = 0, cap = 0, n = 0;
  uint32_t gx = 1, gy = 1, gz = 1;
  int32_t stirAmp = 0;
  uint32_t frame = 0;
  uint64_t substeps = 0;
  bool ballOn = false;
  int32_t ball[3] = {0, 0, 0};
  double ballR = -1.0;
  int32_t reach = 0;
  int32_t bondK = 0, bondBrk = 0;  // build-defined bonds (sn3_write_bonds)
  bool bonds = false;              // some slot of the scene has a bond row
};

struct Engine3 {
  int device = 0, numSMs = 152;
  bool debug = false, chainOn = true;
  uint32_t iters = 3, capSlots = 0, maxCells = 0, maxScenes = 1, matCount = 0;
  std::string err;
  cudaStream_t st = nullptr;
  // the side branch of the substep (inside the captured graph): the cell
  // ranges run on it beside the gather
  cudaStream_t st2 = nullptr;
  cudaEvent_t evFork = nullptr, evJoin = nullptr;
  Bufs3 b{};
  std::vector<int32_t> hluts;
  std::vector<int32_t> hmats;
  std::vector<Scene3Host> sh;
  std::vector<Scene3> hpar;
  World3 hw{};
  uint32_t *tmpK = nullptr, *tmpV = nullptr, *hist = nullptr, *accTmp = nullptr, *fnvBuf = nullptr;
  int2* ballDev = nullptr;
  bool layoutDirty = true, graphValid = false, useGraph = true, anyStir = false;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  uint64_t lastLaunches = 0, launchesPerSubstep = 0;
  cudaEvent_t* pev = nullptr;
  int npev = 0;

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
    return fail("cuda %s: %s", what, cudaGetErrorString(e));
  }

  ~Engine3() {
    if (gexec) cudaGraphExecDestroy(gexec);
    if (graph) cudaGraphDestroy(graph);
    void* ptrs[] = {b.state, b.sceneOf, b.bond, b.bflag, b.inv, b.PRS, b.keys, b.skey, b.sslot, b.cellStart, b.PW, b.PW2, b.PL, b.NBR,
                    b.NBRN, (void*)b.WG, (void*)b.PG, (void*)b.mats, (void*)b.rcp, b.scenes, b.world, b.acc,
                    b.accLast, b.chain, b.dbg, tmpK, tmpV, hist, accTmp, fnvBuf, ballDev, upl, uplRes};
    for (void* p : ptrs)
      if (p) cudaFree(p);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (evFork) cudaEventDestroy(evFork);
    if (evJoin) cudaEventDestroy(evJoin);
    if (st2) cudaStreamDestroy(st2);
    if (st) cudaStreamDestroy(st);
  }

  bool init(const sn3_opts* o) {
    if (!o) return fail("opts is NULL");
    if (o->max_particles == 0) return fail("max_particles must be > 0");
    if (o->max_particles > (1u << 26)) return fail("max_particles above 2^26");
    if (o->iters < 1 || o->iters > 16) return fail("iters = %u outside 1..16", o->iters);
    if (!o->luts || !o->mats) return fail("luts and mats are required");
    if (o->mat_count < 1 || o->mat_count > MAT3_MAX) return fail("mat_count must be 1..%u", MAT3_MAX);
    maxScenes = o->max_scenes ? o->max_scenes : 1;
    if (o->lanes != 0 && o->lanes != 1 && o->lanes != 2 && o->lanes != 4) return fail("lanes must be 0, 1, 2 or 4");
    lanesPin = (int)o->lanes;
    if (maxScenes > (1u << 19)) return fail("max_scenes above 2^19");
    for (uint32_t m = 0; m < o->mat_count; ++m) {
      int32_t rhoW = o->mats[m * 4 + 1];
      if (rhoW < -256 || rhoW > 3839) return fail("mats[%u].rhoW = %d outside -256..3839", m, rhoW);
    }
    device = o->device;
    if (!cuda_ok(cudaSetDevice(device), "cudaSetDevice")) return false;
    cudaDeviceGetAttribute(&numSMs, cudaDevAttrMultiProcessorCount, device);
    debug = o->debug != 0;
    chainOn = o->chain != 0;
    iters = o->iters;
    capSlots = o->max_particles;
    maxCells = o->max_cells ? o->max_cells : (1u << 20);
    matCount = o->mat_count;
    hluts.assign(o->luts, o->luts + LUT_WORDS);
    hmats.assign(o->mats, o->mats + 4 * matCount);
    if (!cuda_ok(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "stream")) return false;
    if (!cuda_ok(cudaStreamCreateWithFlags(&st2, cudaStreamNonBlocking), "stream")) return false;
    cudaEventCreate(&ev0);
    cudaEventCreate(&ev1);
    cudaEventCreateWithFlags(&evFork, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&evJoin, cudaEventDisableTiming);
    size_t C = capSlots;
    b.state = dalloc3<int32_t>(C * 8, err);
    b.sceneOf = dalloc3<uint32_t>(C, err);
    b.bond = dalloc3<uint32_t>(C * BOND3_WORDS, err);
    b.bflag = dalloc3<uint32_t>(C, err);
    b.inv = dalloc3<uint32_t>(C, err);
    b.PRS = dalloc3<int4>(C, err);
    b.keys = dalloc3<uint32_t>(C, err);
    b.skey = dalloc3<uint32_t>(C, err);
    b.sslot = dalloc3<uint32_t>(C, err);
    b.cellStart = dalloc3<uint32_t>((size_t)maxCells + 2, err);
    b.PW = dalloc3<int4>(C, err);
    b.PW2 = dalloc3<int4>(C, err);
    b.PL = dalloc3<int4>(C, err);
    b.NBR = dalloc3<uint32_t>(C * MAXNBR, err);
    b.NBRN = dalloc3<uint32_t>(C, err);
    b.nbrStride = (uint32_t)C;
    int2* dwg = dalloc3<int2>(LUT_N, err);
    int2* dpg = dalloc3<int2>(PLANE_N, err);
    int32_t* dm = dalloc3<int32_t>(4 * matCount, err);
    uint16_t* drcp = dalloc3<uint16_t>(32768, err);
    ballDev = dalloc3<int2>((size_t)maxScenes * BALL_N, err);
    b.scenes = dalloc3<Scene3>(maxScenes, err);
    b.world = dalloc3<World3>(1, err);
    b.acc = dalloc3<uint32_t>((size_t)maxScenes * 8, err);
    b.accLast = dalloc3<uint32_t>((size_t)maxScenes * 8, err);
    b.chain = dalloc3<uint32_t>((size_t)maxScenes * 8, err);
    b.dbg = dalloc3<uint32_t>(16, err);
    tmpK = dalloc3<uint32_t>(C, err);
    tmpV = dalloc3<uint32_t>(C, err);
    hist = dalloc3<uint32_t>(radix::hist_words((uint32_t)C), err);
    accTmp = dalloc3<uint32_t>((size_t)maxScenes * 8, err);
    fnvBuf = dalloc3<uint32_t>(256, err);
    if (!err.empty()) return false;
    {
      std::vector<int2> wg(LUT_N), pg(PLANE_N);
      for (int i = 0; i < LUT_N; ++i) wg[i] = make_int2(o->luts[i], o->luts[LUT_N + i]);
      for (int i = 0; i < PLANE_N; ++i) pg[i] = make_int2(o->luts[2 * LUT_N + i], o->luts[2 * LUT_N + PLANE_N + i]);
      cudaMemcpy(dwg, wg.data(), sizeof(int2) * LUT_N, cudaMemcpyHostToDevice);
      cudaMemcpy(dpg, pg.data(), sizeof(int2) * PLANE_N, cudaMemcpyHostToDevice);
      std::vector<uint16_t> rc(32768);
      for (uint32_t dn = 32768; dn < 65536; ++dn) rc[dn - 32768] = (uint16_t)((1u << 30) / dn);
      cudaMemcpy(drcp, rc.data(), 65536, cudaMemcpyHostToDevice);
      cudaMemcpy(dm, hmats.data(), sizeof(int32_t) * hmats.size(), cudaMemcpyHostToDevice);
    }
    b.WG = dwg;
    b.PG = dpg;
    b.mats = dm;
    b.rcp = drcp;
    b.BALL = ballDev;
    sh.assign(maxScenes, Scene3Host{});
    hpar.assign(maxScenes, Scene3{});
    return cuda_ok(cudaDeviceSynchronize(), "init");
  }

  // buildBallLUT (3d/app.js:212-230) in IEEE double arithmetic, the same
  // operations in the same order, so the tables are bit-identical.
  void ball_tables(double R, std::vector<int2>& out) const {
    const int32_t* planeW = hluts.data() + 2 * LUT_N;
    const int32_t* planeG = planeW + PLANE_N;
    out.assign(BALL_N, make_int2(0, 0));
    for (int bi = 0; bi < BALL_N; ++bi) {
      double r = std::sqrt((double)bi * 4096.0) / 256.0;
      double depth = r - R;
      if (depth >= 2.0) continue;
      double d = std::max(depth, 0.0);
      double at = js_round(d * 256.0);
      int idx = (int)std::max(0.0, std::min(512.0, at));
      int32_t g = 0;
      if (r > 1e-6) g = (int32_t)std::min(js_round((double)planeG[idx] / r), (double)(1 << 24));
      out[bi] = make_int2(planeW[idx], g);
    }
  }

  // Lanes per particle in the density and solve gathers (results do not
  // depend on them), and resident CTAs per SM per kernel for one-wave grids.
  int lanesD = 1, lanesS = 1, lanesN = 1, lanesPin = 0;
  bool lanesTuned = false;
  std::vector<std::pair<const void*, int>> occCache;
  int grid_occ(const void* k, uint64_t items) {
    int nb = 0;
    for (auto& kv : occCache)
      if (kv.first == k) nb = kv.second;
    if (!nb) {
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, 256, 0) != cudaSuccess || nb < 1) nb = 1;
      occCache.push_back({k, nb});
    }
    uint64_t g = (items + 255) / 256;
    return (int)std::max<uint64_t>(1, std::min<uint64_t>(g, (uint64_t)numSMs * nb));
  }
  void default_lanes() {
    if (lanesPin) {
      lanesD = lanesS = lanesN = lanesPin;
      return;
    }
    if (lanesTuned) return;
    // Measured on 3D columns (ms per substep with 1 / 2 / 4 lanes): 32,768
    // particles 0.162 / 0.141 / 0.119, 64,000 0.183 / 0.179 / 0.166,
    // 85,184 0.209 / 0.211 / 0.206, 97,336 0.226 / 0.237 / 0.238, 262,144
    // 0.387 / 0.500 / 0.531: two lanes never won.
    const uint32_t n = hw.nAct;
    lanesD = lanesS = n < 90112 ? 4 : 1;
    lanesN = 1;  // the ballot-split list build measured slower than one lane per particle
  }

  uint32_t grid_for(uint32_t n) const {
    uint32_t g = (n + 255) / 256;
    return std::max(1u, std::min(g, (uint32_t)numSMs * 64u));
  }

  bool relayout() {
    uint32_t K = 0, slotEnd = 0, nAct = 0, numScenes = 0;
    anyStir = false;
    for (uint32_t s = 0; s < maxScenes; ++s) {
      Scene3Host& h = sh[s];
      Scene3 p{};
      if (h.used) {
        numScenes = s + 1;
        slotEnd = std::max(slotEnd, h.slotBase + h.cap);
      }
      if (h.used && h.loaded) {
        p.slotBase = h.slotBase;
        p.cap = h.cap;
        p.n = h.n;
        p.keyOff = K;
        p.gx = h.gx;
        p.gy = h.gy;
        p.gz = h.gz;
        p.cellTotal = h.gx * h.gy * h.gz;
        p.wmax[0] = (int32_t)h.gx * H;
        p.wmax[1] = (int32_t)h.gy * H;
        p.wmax[2] = (int32_t)h.gz * H;
        p.stirPhase = (int32_t)((h.substeps * 384ull) & 131071ull);
        p.stirAmp = h.stirAmp;
        p.substep = (uint32_t)h.substeps;
        p.frame = h.frame;
        p.ballOn = h.ballOn ? 1u : 0u;
        p.ball[0] = h.ball[0];
        p.ball[1] = h.ball[1];
        p.ball[2] = h.ball[2];
        p.reach = h.reach;
        p.bondK = h.bondK;
        p.bondBrk = h.bondBrk;
        p.active = 1;
        K += p.cellTotal;
        nAct += h.n;
        anyStir |= h.stirAmp != 0;
      }
      hpar[s] = p;
    }
    if (K > maxCells) return fail("the scenes need %u grid cells, above max_cells = %u", K, maxCells);
    hw = World3{numScenes, K, slotEnd, nAct};
    default_lanes();
    std::vector<uint32_t> sceneOf(std::max(slotEnd, 1u), NO_SCENE);
    for (uint32_t s = 0; s < maxScenes; ++s)
      if (sh[s].used && sh[s].loaded)
        for (uint32_t i = 0; i < sh[s].cap; ++i) sceneOf[sh[s].slotBase + i] = s;
    cudaMemcpyAsync(b.sceneOf, sceneOf.data(), sizeof(uint32_t) * sceneOf.size(), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(b.scenes, hpar.data(), sizeof(Scene3) * maxScenes, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(b.world, &hw, sizeof(World3), cudaMemcpyHostToDevice, st);
    if (!cuda_ok(cudaStreamSynchronize(st), "relayout")) return false;
    layoutDirty = false;
    graphValid = false;
    return true;
  }

  void mark(int* count) {
    if (pev) cudaEventRecord(pev[npev++], st);
    if (count) ++*count;
  }

  template <bool DBG>
  void launch_t() {
    const uint32_t gS = grid_for(hw.slotEnd), gA = grid_for(hw.nAct), gK = grid_for(hw.K + 1);
    int launches = 0;
    mark(nullptr);
    k3_predict<DBG><<<gS, 256, 0, st>>>(b);
    ++launches;
    mark(nullptr);
    int keyBits = 32 - __builtin_clz(std::max(hw.K, 1u));
    radix::sort_pairs(b.keys, hw.slotEnd, keyBits, b.skey, b.sslot, tmpK, tmpV, hist, st);
    launches += radix::LAUNCHES_PER_PASS * std::max(1, (keyBits + radix::RBITS - 1) / radix::RBITS);
    mark(nullptr);
    cudaEventRecord(evFork, st);
    cudaStreamWaitEvent(st2, evFork, 0);
    k3_cellstart<<<gK, 256, 0, st2>>>(b);
    cudaEventRecord(evJoin, st2);
    k3_gather<<<gA, 256, 0, st>>>(b);
    cudaStreamWaitEvent(st, evJoin, 0);
    launches += 2;
    mark(nullptr);
    switch (lanesN) {
      case 4: k3_nbr<DBG, 4><<<grid_occ((const void*)k3_nbr<DBG, 4>, (uint64_t)hw.nAct * 4), 256, 0, st>>>(b); break;
      case 2: k3_nbr<DBG, 2><<<grid_occ((const void*)k3_nbr<DBG, 2>, (uint64_t)hw.nAct * 2), 256, 0, st>>>(b); break;
      default: k3_nbr<DBG, 1><<<grid_occ((const void*)k3_nbr<DBG, 1>, hw.nAct), 256, 0, st>>>(b); break;
    }
    ++launches;
    mark(nullptr);
    int4* cur = b.PW;
    int4* nxt = b.PW2;
    for (uint32_t it = 0; it < iters; ++it) {
      switch (lanesD) {
        case 4: k3_density<DBG, 4><<<grid_occ((const void*)k3_density<DBG, 4>, (uint64_t)hw.nAct * 4), 256, 0, st>>>(b, cur); break;
        case 2: k3_density<DBG, 2><<<grid_occ((const void*)k3_density<DBG, 2>, (uint64_t)hw.nAct * 2), 256, 0, st>>>(b, cur); break;
        default: k3_density<DBG, 1><<<grid_occ((const void*)k3_density<DBG, 1>, hw.nAct), 256, 0, st>>>(b, cur); break;
      }
      mark(nullptr);
      switch (lanesS) {
        case 4: k3_solve<DBG, 4><<<grid_occ((const void*)k3_solve<DBG, 4>, (uint64_t)hw.nAct * 4), 256, 0, st>>>(b, cur, nxt); break;
        case 2: k3_solve<DBG, 2><<<grid_occ((const void*)k3_solve<DBG, 2>, (uint64_t)hw.nAct * 2), 256, 0, st>>>(b, cur, nxt); break;
        default: k3_solve<DBG, 1><<<grid_occ((const void*)k3_solve<DBG, 1>, hw.nAct), 256, 0, st>>>(b, cur, nxt); break;
      }
      mark(nullptr);
      std::swap(cur, nxt);
      launches += 2;
    }
    if (chainOn) k3_integrate<DBG, true><<<gA, 256, 0, st>>>(b, cur);
    else k3_integrate<DBG, false><<<gA, 256, 0, st>>>(b, cur);
    mark(nullptr);
    k3_fold<<<(hw.numScenes + 63) / 64, 64, 0, st>>>(b, chainOn ? 1 : 0);
    launches += 2;
    mark(nullptr);
    launchesPerSubstep = (uint64_t)launches;
  }
  void launch_one() {
    if (debug) launch_t<true>(); else launch_t<false>();
  }

  bool any_loaded() const {
    for (auto& s : sh)
      if (s.used && s.loaded) return true;
    return false;
  }

  // runSubsteps (3d/app.js:709-714): the stir phase is written once per call.
  bool upload_phase() {
    for (uint32_t s = 0; s < maxScenes; ++s)
      if (sh[s].used && sh[s].loaded) {
        hpar[s].stirPhase = (int32_t)((sh[s].substeps * 384ull) & 131071ull);
        hpar[s].substep = (uint32_t)sh[s].substeps;
      }
    return cuda_ok(cudaMemcpyAsync(b.scenes, hpar.data(), sizeof(Scene3) * hw.numScenes, cudaMemcpyHostToDevice, st),
                   "params");
  }

  bool step(uint32_t count) {
    if (!any_loaded()) return fail("step() called before a scene was loaded");
    if (count == 0) return true;
    if (layoutDirty && !relayout()) return false;
    if (anyStir && !upload_phase()) return false;
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
    accFresh = chainOn;
    return cuda_ok(cudaGetLastError(), "step");
  }

  // Phases: predict, sort, cellstart+gather, nbr, then (density, solve) per
  // iteration, integrate(+hash), fold.
  bool profile(uint32_t reps, float* out, uint32_t maxOut, uint32_t* nOut) {
    if (!any_loaded()) return fail("profile before a scene was loaded");
    if (layoutDirty && !relayout()) return false;
    if (anyStir && !upload_phase()) return false;
    const int NE = 8 + 2 * (int)iters + 4;
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
      accFresh = chainOn;
    }
    for (auto& e : evs) cudaEventDestroy(e);
    uint32_t n = (uint32_t)std::max(0, used - 1);
    for (uint32_t k = 0; k < n && k < maxOut; ++k) out[k] = (float)(acc[k] / std::max(1u, reps));
    if (nOut) *nOut = n;
    return true;
  }

  bool check_scene(uint32_t s, bool needLoaded = true) {
    if (s >= maxScenes || !sh[s].used) return fail("no scene %u", s);
    if (needLoaded && !sh[s].loaded) return fail("scene %u is not loaded", s);
    return true;
  }

  bool alloc_scene(uint32_t cap, uint32_t* id) {
    uint32_t s = 0;
    while (s < maxScenes && sh[s].used) ++s;
    if (s == maxScenes) return fail("all %u scene slots are in use", maxScenes);
    if (cap == 0) return fail("scene capacity must be > 0");
    std::vector<std::pair<uint32_t, uint32_t>> usedR;
    for (auto& h : sh)
      if (h.used) usedR.push_back({h.slotBase, h.slotBase + h.cap});
    std::sort(usedR.begin(), usedR.end());
    uint32_t base = 0;
    bool found = false;
    for (auto& r : usedR) {
      if (r.first >= base + (uint64_t)cap) { found = true; break; }
      base = std::max(base, r.second);
    }
    if (!found && (uint64_t)base + cap > capSlots) return fail("no room for %u slots", cap);
    sh[s] = Scene3Host{};
    sh[s].used = true;
    sh[s].slotBase = base;
    sh[s].cap = cap;
    *id = s;
    layoutDirty = true;
    return true;
  }

  bool load(uint32_t s, const sn3_scene* sc) {
    accFresh = false;
    if (!check_scene(s, false)) return false;
    if (!sc) return fail("scene is NULL");
    Scene3Host& h = sh[s];
    if (sc->n > h.cap) return fail("scene has %u particles, above this scene's capacity %u", sc->n, h.cap);
    if (sc->n > 0 && (!sc->pos || !sc->mat)) return fail("pos and mat are required");
    for (uint32_t a : {sc->gx, sc->gy, sc->gz})
      if (a < 1 || a > MAX_AXIS_CELLS) return fail("grid dims must be 1..%u cells per axis", MAX_AXIS_CELLS);
    // the arrays go up as they are (pos 3n, vel 3n, mat n), are checked on the
    // device (the first bad material index) and packed there; a refused load
    // leaves the scene's state as it was
    if (sc->n) {
      if (!ensure_upload()) return false;
      const size_t n = sc->n;
      bool ok = cuda_ok(cudaMemcpyAsync(upl, sc->pos, n * 12, cudaMemcpyHostToDevice, st), "upload") &&
                (!sc->vel || cuda_ok(cudaMemcpyAsync(upl + 3 * n, sc->vel, n * 12, cudaMemcpyHostToDevice, st), "upload")) &&
                cuda_ok(cudaMemcpyAsync(upl + 6 * n, sc->mat, n * 4, cudaMemcpyHostToDevice, st), "upload");
      const uint32_t none = 0xffffffffu;
      ok = ok && cuda_ok(cudaMemcpyAsync(uplRes, &none, 4, cudaMemcpyHostToDevice, st), "upload");
      if (!ok) return false;
      k3_load_check<<<grid_for(sc->n), 256, 0, st>>>(upl, sc->n, matCount, uplRes);
      uint32_t bad = 0;
      cudaMemcpyAsync(&bad, uplRes, 4, cudaMemcpyDeviceToHost, st);
      if (!cuda_ok(cudaStreamSynchronize(st), "load check")) return false;
      if (bad != none) return fail("mat[%u] = %u outside the material table", bad, sc->mat[bad]);
      k3_load_pack<<<grid_for(sc->n), 256, 0, st>>>(upl, sc->n, sc->vel ? 1u : 0u, b.state + (size_t)h.slotBase * 8);
      if (!cuda_ok(cudaGetLastError(), "pack")) return false;
    }
    static const uint32_t CHAIN_INIT[8] = {0x243f6a88u, 0x85a308d3u, 0x13198a2eu, 0x03707344u,
                                           0xa4093822u, 0x299f31d0u, 0x082efa98u, 0xec4e6c89u};
    cudaMemcpyAsync(b.chain + (size_t)s * 8, CHAIN_INIT, 32, cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(b.acc + (size_t)s * 8, 0, 32, st);
    if (!clear_bonds(s)) return false;
    h.n = sc->n;
    h.gx = sc->gx;
    h.gy = sc->gy;
    h.gz = sc->gz;
    h.stirAmp = sc->stir_amp;
    h.frame = sc->frame;
    h.substeps = 0;
    h.loaded = true;
    layoutDirty = true;
    return cuda_ok(cudaStreamSynchronize(st), "load");
  }

  // A device buffer the scene loads and bond writes upload into before their
  // device-side checks (capSlots x BOND3_WORDS words: fits either).
  int32_t* upl = nullptr;
  uint32_t* uplRes = nullptr;
  bool ensure_upload() {
    if (upl) return true;
    upl = dalloc3<int32_t>((size_t)capSlots * BOND3_WORDS, err);
    uplRes = dalloc3<uint32_t>(2, err);
    return upl && uplRes;
  }

  bool clear_bonds(uint32_t s) {
    Scene3Host& h = sh[s];
    h.bonds = false;
    h.bondK = h.bondBrk = 0;
    return cuda_ok(cudaMemsetAsync(b.bond + (size_t)h.slotBase * BOND3_WORDS, 0, (size_t)h.cap * BOND3_WORDS * 4, st),
                   "bonds") &&
           cuda_ok(cudaMemsetAsync(b.bflag + h.slotBase, 0, (size_t)h.cap * 4, st), "bonds");
  }

  // Bond rows of scene s (BOND3_CAP entries of {partner + 1, L0} per particle,
  // scene-local partner indices, each bond in both ends' rows), with the
  // scene's stiffness and break ratio. Build-defined: the reference's 3D page
  // has no bonds.
  bool write_bonds(uint32_t s, const uint32_t* rows, size_t words, int32_t k, int32_t brk) {
    accFresh = false;
    if (!check_scene(s)) return false;
    Scene3Host& h = sh[s];
    if (!rows || words != (size_t)h.n * BOND3_WORDS) return fail("bond rows need n * %u words", BOND3_WORDS);
    if (k < 0 || k > 65536) return fail("bond stiffness %d outside 0..65536", k);
    if (brk < 0) return fail("bond break ratio must be >= 0");
    // the rows go up as they are and are checked on the device (the first bad
    // row is then named by the same host rules); a refused write leaves the
    // scene's rows as they were
    if (!ensure_upload()) return false;
    const uint32_t none[2] = {0xffffffffu, 0u};
    bool ok = cuda_ok(cudaMemcpyAsync(upl, rows, words * 4, cudaMemcpyHostToDevice, st), "upload") &&
              cuda_ok(cudaMemcpyAsync(uplRes, none, 8, cudaMemcpyHostToDevice, st), "upload");
    if (!ok) return false;
    if (h.n) k3_bonds_check<<<grid_for(h.n), 256, 0, st>>>(reinterpret_cast<const uint32_t*>(upl), h.n, uplRes);
    uint32_t res[2];
    cudaMemcpyAsync(res, uplRes, 8, cudaMemcpyDeviceToHost, st);
    if (!cuda_ok(cudaStreamSynchronize(st), "bond check")) return false;
    if (res[0] != 0xffffffffu) {
      const uint32_t i = res[0];
      const uint32_t* r = rows + (size_t)i * BOND3_WORDS;
      bool ended = false;
      for (uint32_t e = 0; e < BOND3_CAP; ++e) {
        const uint32_t w = r[2 * e], L0 = r[2 * e + 1];
        if (w == 0u) {
          ended = true;
          if (L0 != 0u) return fail("bond row %u: an empty entry carries a rest length", i);
          continue;
        }
        if (ended) return fail("bond row %u: an entry follows the end of the row", i);
        const uint32_t j = (w & BOND3_J) - 1u;
        if (j >= h.n || j == i) return fail("bond row %u names partner %u", i, j);
        if ((int32_t)L0 < BOND3_L0_MIN || (int32_t)L0 > BOND3_L0_MAX)
          return fail("bond row %u: rest length %u outside %d..%d", i, L0, BOND3_L0_MIN, BOND3_L0_MAX);
      }
      return fail("bond row %u failed the device check but passes the host check", i);
    }
    const bool any = res[1] != 0u;
    if (!clear_bonds(s)) return false;
    if (h.n) {
      cudaMemcpyAsync(b.bond + (size_t)h.slotBase * BOND3_WORDS, upl, words * 4, cudaMemcpyDeviceToDevice, st);
      k3_bond_flags<<<grid_for(h.n), 256, 0, st>>>(b.bond + (size_t)h.slotBase * BOND3_WORDS, h.n,
                                                     b.bflag + h.slotBase);
    }
    h.bonds = any;
    h.bondK = k;
    h.bondBrk = brk;
    layoutDirty = true;
    return cuda_ok(cudaStreamSynchronize(st), "write_bonds");
  }

  bool read_bonds(uint32_t s, uint32_t* out, size_t words) {
    if (!check_scene(s)) return false;
    const size_t need = (size_t)sh[s].n * BOND3_WORDS;
    if (!out || words < need) return fail("read_bonds needs %zu words", need);
    cudaMemcpyAsync(out, b.bond + (size_t)sh[s].slotBase * BOND3_WORDS, need * 4, cudaMemcpyDeviceToHost, st);
    return cuda_ok(cudaStreamSynchronize(st), "read_bonds");
  }

  bool remove(uint32_t s) {
    if (!check_scene(s, false)) return false;
    if (!clear_bonds(s) || !cuda_ok(cudaStreamSynchronize(st), "remove")) return false;
    sh[s] = Scene3Host{};
    layoutDirty = true;
    return true;
  }

  // spawn (3d/app.js:575-597): append up to k particles (velocity zero) past
  // the scene's live count; what does not fit the capacity is dropped.
  bool spawn(uint32_t s, const int32_t* pos, const uint32_t* mat, uint32_t k, uint32_t* added) {
    accFresh = false;
    if (!check_scene(s)) return false;
    if (k > 0 && (!pos || !mat)) return fail("pos and mat are required");
    Scene3Host& h = sh[s];
    uint32_t room = h.cap - h.n;
    if (k > room) k = room;
    for (uint32_t i = 0; i < k; ++i)
      if (mat[i] >= matCount) return fail("mat[%u] = %u outside the material table", i, mat[i]);
    if (k > 0) {
      std::vector<int32_t> words((size_t)k * 8, 0);
      for (uint32_t i = 0; i < k; ++i) {
        int32_t* w = words.data() + (size_t)i * 8;
        w[0] = pos[3 * i];
        w[1] = pos[3 * i + 1];
        w[2] = pos[3 * i + 2];
        w[3] = (int32_t)mat[i];
      }
      cudaMemcpyAsync(b.state + (size_t)(h.slotBase + h.n) * 8, words.data(), words.size() * 4,
                      cudaMemcpyHostToDevice, st);
      if (!cuda_ok(cudaStreamSynchronize(st), "spawn")) return false;
      h.n += k;
      layoutDirty = true;
    }
    if (added) *added = k;
    return true;
  }

  bool set_ball(uint32_t s, uint32_t on, int32_t x, int32_t y, int32_t z, double R) {
    if (!check_scene(s, false)) return false;
    if (!(R > 0.0 && R <= 64.0)) return fail("ball radius must be in (0, 64] world units");
    Scene3Host& h = sh[s];
    if (R != h.ballR) {
      std::vector<int2> tab;
      ball_tables(R, tab);
      cudaMemcpyAsync(ballDev + (size_t)s * BALL_N, tab.data(), sizeof(int2) * BALL_N, cudaMemcpyHostToDevice, st);
      if (!cuda_ok(cudaStreamSynchronize(st), "ball")) return false;
      h.ballR = R;
    }
    h.ballOn = on != 0;
    h.ball[0] = x;
    h.ball[1] = y;
    h.ball[2] = z;
    h.reach = (int32_t)js_round((R + 2.0) * ONE);
    layoutDirty = true;
    return true;
  }

  // accFresh: the fold's last digest is the digest of the current state (set
  // by stepping with the chain on, cleared by any change made outside a substep).
  bool accFresh = false;
  bool digest(uint32_t s, uint32_t out[8]) {
    if (!check_scene(s)) return false;
    if (accFresh && !layoutDirty) {
      cudaMemcpyAsync(out, b.accLast + (size_t)s * 8, 32, cudaMemcpyDeviceToHost, st);
      return cuda_ok(cudaStreamSynchronize(st), "digest");
    }
    if (layoutDirty && !relayout()) return false;
    cudaMemsetAsync(accTmp, 0, sizeof(uint32_t) * 8 * maxScenes, st);
    k3_hash<<<grid_for(hw.slotEnd), 256, 0, st>>>(b, accTmp);
    cudaMemcpyAsync(out, accTmp + s * 8, 32, cudaMemcpyDeviceToHost, st);
    return cuda_ok(cudaStreamSynchronize(st), "digest");
  }

  // chain() (3d/app.js:717-744): stripe words on the device, the 8-lane fold
  // on the host in index order.
  bool fnv(uint32_t s, uint32_t out[8]) {
    if (!check_scene(s)) return false;
    uint32_t words[256];
    k3_fnv<<<1, 256, 0, st>>>(b.state, sh[s].slotBase, sh[s].n, fnvBuf);
    cudaMemcpyAsync(words, fnvBuf, sizeof(words), cudaMemcpyDeviceToHost, st);
    if (!cuda_ok(cudaStreamSynchronize(st), "fnv")) return false;
    for (uint32_t L = 0; L < 8; ++L) out[L] = 2166136261u ^ (L * 0x9e3779b9u);
    for (uint32_t k = 0; k < 256; ++k)
      for (uint32_t L = 0; L < 8; ++L) {
        uint32_t v = (out[L] ^ words[k]) * 16777619u;
        out[L] = v ^ (v >> 13);
      }
    return true;
  }

  bool chain(uint32_t s, uint32_t out[8]) {
    if (!check_scene(s)) return false;
    cudaMemcpyAsync(out, b.chain + (size_t)s * 8, 32, cudaMemcpyDeviceToHost, st);
    return cuda_ok(cudaStreamSynchronize(st), "chain");
  }

  bool read_state(uint32_t s, int32_t* out, size_t words) {
    if (!check_scene(s)) return false;
    size_t need = (size_t)sh[s].n * 8;
    if (!out || words < need) return fail("read_state needs %zu words", need);
    cudaMemcpyAsync(out, b.state + (size_t)sh[s].slotBase * 8, need * 4, cudaMemcpyDeviceToHost, st);
    return cuda_ok(cudaStreamSynchronize(st), "read_state");
  }

  // A keyframe: the state words fully determine every later substep (the
  // solver's other fields are rewritten before they are read), plus the
  // substep count (for the stir phase) and the chain.
  bool write_state(uint32_t s, const int32_t* state, uint32_t n, uint64_t substeps, const uint32_t* chainIn) {
    accFresh = false;
    if (!check_scene(s)) return false;
    Scene3Host& h = sh[s];
    if (n > h.cap) return fail("state has %u particles, above capacity %u", n, h.cap);
    if (n > 0 && !state) return fail("state is NULL");
    for (uint32_t i = 0; i < n; ++i)
      if ((uint32_t)state[(size_t)i * 8 + 3] >= matCount) return fail("state row %u names no material", i);
    if (n > 0)
      cudaMemcpyAsync(b.state + (size_t)h.slotBase * 8, state, (size_t)n * 32, cudaMemcpyHostToDevice, st);
    if (chainIn) cudaMemcpyAsync(b.chain + (size_t)s * 8, chainIn, 32, cudaMemcpyHostToDevice, st);
    if (!cuda_ok(cudaStreamSynchronize(st), "write_state")) return false;
    h.n = n;
    h.substeps = substeps;
    layoutDirty = true;
    return true;
  }

  // Device checkpoint of scene s: [state n*8][chain 8] and the substep clock.
  size_t ckpt_bytes(uint32_t s) const { return (size_t)sh[s].n * 32 + 32; }
  bool ckpt_save(uint32_t s, sn_ckpt_pool* pool, uint64_t* handle) {
    if (!check_scene(s)) return false;
    if (pool->device != device) return fail("checkpoint pool is on device %d, the engine on %d", pool->device, device);
    const Scene3Host& h = sh[s];
    sn_ckpt_pool::Rec* r = nullptr;
    if (!pool->reserve(ckpt_bytes(s), 3, handle, &r)) return fail("%s", pool->err.c_str());
    char* d = pool->base + r->off;
    bool ok = cuda_ok(cudaMemcpyAsync(d, b.state + (size_t)h.slotBase * 8, (size_t)h.n * 32, cudaMemcpyDeviceToDevice,
                                      st), "ckpt") &&
              cuda_ok(cudaMemcpyAsync(d + (size_t)h.n * 32, b.chain + (size_t)s * 8, 32, cudaMemcpyDeviceToDevice, st),
                      "ckpt");
    r->n = h.n;
    r->substeps = h.substeps;
    cudaEventRecord(r->done, st);
    if (!ok) {
      pool->free_rec(*handle);
      return false;
    }
    return true;
  }
  bool ckpt_load(uint32_t s, sn_ckpt_pool* pool, uint64_t handle) {
    accFresh = false;
    if (!check_scene(s)) return false;
    sn_ckpt_pool::Rec* r = pool->find(handle);
    if (!r || r->kind != 3) return fail("no 3D checkpoint %llu in the pool", (unsigned long long)handle);
    Scene3Host& h = sh[s];
    if (r->n > h.cap) return fail("checkpoint holds %u particles, above this scene's capacity %u", r->n, h.cap);
    cudaStreamWaitEvent(st, r->done, 0);
    const char* d = pool->base + r->off;
    bool ok = cuda_ok(cudaMemcpyAsync(b.state + (size_t)h.slotBase * 8, d, (size_t)r->n * 32, cudaMemcpyDeviceToDevice,
                                      st), "load") &&
              cuda_ok(cudaMemcpyAsync(b.chain + (size_t)s * 8, d + (size_t)r->n * 32, 32, cudaMemcpyDeviceToDevice, st),
                      "load");
    cudaEventRecord(r->done, st);
    if (!ok) return false;
    if (h.n != r->n) layoutDirty = true;
    h.n = r->n;
    h.substeps = r->substeps;
    // the device copy of the substep clock follows the host one
    hpar[s].substep = (uint32_t)h.substeps;
    hpar[s].stirPhase = (int32_t)((h.substeps * 384ull) & 131071ull);
    if (!layoutDirty &&
        !cuda_ok(cudaMemcpyAsync(b.scenes + s, &hpar[s], sizeof(Scene3), cudaMemcpyHostToDevice, st), "load"))
      return false;
    return cuda_ok(cudaStreamSynchronize(st), "load");
  }

  bool timing(float* ms) {
    if (!cuda_ok(cudaEventSynchronize(ev1), "timing")) return false;
    cudaEventElapsedTime(ms, ev0, ev1);
    return true;
  }
};

}  // namespace

struct sn3_engine {
  Engine3 w;
};

static int rc3(Engine3& w, bool ok) {
  if (ok) return SN_OK;
  return w.err.rfind("cuda", 0) == 0 ? SN_E_CUDA : SN_E_INVALID;
}

extern "C" {

int sn3_create(const sn3_opts* opts, sn3_engine** out) {
  if (!out) return SN_E_INVALID;
  *out = nullptr;
  sn3_engine* e = new sn3_engine();
  if (!e->w.init(opts)) {
    fprintf(stderr, "[suna3d] create: %s\n", e->w.err.c_str());
    delete e;
    return SN_E_INVALID;
  }
  *out = e;
  return SN_OK;
}
void sn3_destroy(sn3_engine* e) { delete e; }
const char* sn3_last_error(const sn3_engine* e) { return e ? e->w.err.c_str() : "null engine"; }

int sn3_load_scene(sn3_engine* e, const sn3_scene* sc) {
  if (!e) return SN_E_INVALID;
  Engine3& w = e->w;
  for (uint32_t s = 0; s < w.maxScenes; ++s)
    if (w.sh[s].used) w.remove(s);
  uint32_t id = 0;
  if (!w.alloc_scene(w.capSlots, &id)) return SN_E_CAPACITY;
  bool ok = w.load(id, sc);
  if (!ok) w.remove(id);
  return rc3(w, ok);
}
int sn3_add_scene(sn3_engine* e, const sn3_scene* sc, uint32_t cap, uint32_t* scene_out) {
  if (!e || !sc) return SN_E_INVALID;
  Engine3& w = e->w;
  uint32_t id = 0;
  if (cap == 0) cap = sc->n;
  if (!w.alloc_scene(cap, &id)) return SN_E_CAPACITY;
  if (!w.load(id, sc)) {
    w.remove(id);
    return SN_E_INVALID;
  }
  if (scene_out) *scene_out = id;
  return SN_OK;
}
int sn3_remove_scene(sn3_engine* e, uint32_t scene) {
  if (!e) return SN_E_INVALID;
  return rc3(e->w, e->w.remove(scene));
}
int sn3_step(sn3_engine* e, uint32_t count) {
  if (!e) return SN_E_INVALID;
  if (!e->w.any_loaded()) {
    e->w.err = "step() called before a scene was loaded";
    return SN_E_STATE;
  }
  return rc3(e->w, e->w.step(count));
}
int sn3_spawn(sn3_engine* e, uint32_t scene, const int32_t* pos, const uint32_t* mat, uint32_t k, uint32_t* added) {
  if (!e) return SN_E_INVALID;
  return rc3(e->w, e->w.spawn(scene, pos, mat, k, added));
}
int sn3_set_ball(sn3_engine* e, uint32_t scene, uint32_t on, int32_t x, int32_t y, int32_t z, double radius_wu) {
  if (!e) return SN_E_INVALID;
  return rc3(e->w, e->w.set_ball(scene, on, x, y, z, radius_wu));
}
int sn3_fnv(sn3_engine* e, uint32_t scene, uint32_t lanes[8]) {
  if (!e || !lanes) return SN_E_INVALID;
  return rc3(e->w, e->w.fnv(scene, lanes));
}
int sn3_digest(sn3_engine* e, uint32_t scene, uint32_t acc[8]) {
  if (!e || !acc) return SN_E_INVALID;
  return rc3(e->w, e->w.digest(scene, acc));
}
int sn3_chain(sn3_engine* e, uint32_t scene, uint32_t chain[8]) {
  if (!e || !chain) return SN_E_INVALID;
  return rc3(e->w, e->w.chain(scene, chain));
}
int sn3_write_bonds(sn3_engine* e, uint32_t scene, const uint32_t* rows, size_t words, int32_t stiffness,
                    int32_t break_ratio) {
  if (!e) return SN_E_INVALID;
  return rc3(e->w, e->w.write_bonds(scene, rows, words, stiffness, break_ratio));
}
int sn3_read_bonds(sn3_engine* e, uint32_t scene, uint32_t* out, size_t words) {
  if (!e) return SN_E_INVALID;
  return rc3(e->w, e->w.read_bonds(scene, out, words));
}
int sn3_read_state(sn3_engine* e, uint32_t scene, int32_t* out, size_t words) {
  if (!e) return SN_E_INVALID;
  return rc3(e->w, e->w.read_state(scene, out, words));
}
int sn3_write_state(sn3_engine* e, uint32_t scene, const int32_t* state, uint32_t n, uint64_t substeps,
                    const uint32_t chain[8]) {
  if (!e) return SN_E_INVALID;
  return rc3(e->w, e->w.write_state(scene, state, n, substeps, chain));
}
int sn3_debug_counters(sn3_engine* e, uint32_t out[16]) {
  if (!e || !out) return SN_E_INVALID;
  cudaMemcpyAsync(out, e->w.b.dbg, 64, cudaMemcpyDeviceToHost, e->w.st);
  return rc3(e->w, e->w.cuda_ok(cudaStreamSynchronize(e->w.st), "debug_counters"));
}
int sn3_sync(sn3_engine* e) {
  if (!e) return SN_E_INVALID;
  return rc3(e->w, e->w.cuda_ok(cudaStreamSynchronize(e->w.st), "sync"));
}
int sn3_get_info(sn3_engine* e, uint32_t scene, sn3_info* out) {
  if (!e || !out) return SN_E_INVALID;
  Engine3& w = e->w;
  if (!w.check_scene(scene, false)) return SN_E_INVALID;
  const Scene3Host& h = w.sh[scene];
  out->n = h.n;
  out->cap = h.cap;
  out->gx = h.gx;
  out->gy = h.gy;
  out->gz = h.gz;
  out->iters = w.iters;
  out->substep_count = h.substeps;
  return SN_OK;
}
int sn3_last_timing(sn3_engine* e, float* ms, uint64_t* launches) {
  if (!e) return SN_E_INVALID;
  if (ms && !e->w.timing(ms)) return SN_E_CUDA;
  if (launches) *launches = e->w.lastLaunches;
  return SN_OK;
}
int sn3_profile_substep(sn3_engine* e, uint32_t reps, float* ms, uint32_t max_phases, uint32_t* n_phases) {
  if (!e || !ms) return SN_E_INVALID;
  return rc3(e->w, e->w.profile(reps, ms, max_phases, n_phases));
}

int sn3_ckpt_bytes(sn3_engine* e, uint32_t scene, size_t* bytes) {
  if (!e || !bytes) return SN_E_INVALID;
  if (!e->w.check_scene(scene)) return SN_E_INVALID;
  *bytes = e->w.ckpt_bytes(scene);
  return SN_OK;
}
int sn3_ckpt_save(sn3_engine* e, uint32_t scene, sn_ckpt_pool* p, uint64_t* handle) {
  if (!e || !p || !handle) return SN_E_INVALID;
  if (e->w.ckpt_save(scene, p, handle)) return SN_OK;
  return e->w.err.rfind("checkpoint pool full", 0) == 0 ? SN_E_CAPACITY : rc3(e->w, false);
}
int sn3_ckpt_load(sn3_engine* e, uint32_t scene, sn_ckpt_pool* p, uint64_t handle) {
  if (!e || !p) return SN_E_INVALID;
  return rc3(e->w, e->w.ckpt_load(scene, p, handle));
}

}  // extern "C"
