// Device checkpoint pool shared by the 2D and 3D engines (sn_ckpt_pool in
// include/suna.h). One device allocation, carved first-fit on the host into
// 256-byte aligned records. Every record carries a CUDA event recorded after
// the last copy that touched it on whichever engine stream made the copy, so a
// load on another stream waits for the save, and freeing a record (or reusing
// its bytes) waits for every copy in flight.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <map>
#include <string>
#include <unordered_map>
#include <vector>

struct sn_ckpt_pool {
  struct Rec {
    size_t off = 0, bytes = 0;
    uint32_t kind = 0;  // 2 = 2D scene, 3 = 3D scene
    uint32_t n = 0, nFluid = 0, hasBonds = 0;
    uint64_t substeps = 0, formClock = 0;
    uint32_t dirty = 0;
    cudaEvent_t done = nullptr;
    // a 2D scene's rigid bodies: their records and driver sidecars travel on
    // the host (a few hundred bytes each), their rest offsets in the pool
    uint32_t nBodies = 0;
    std::vector<int32_t> bodyRec, bodyDrv;
  };
  int device = 0;
  char* base = nullptr;
  size_t cap = 0, used = 0;
  std::string err;
  std::map<size_t, size_t> freeList;  // offset -> bytes
  std::unordered_map<uint64_t, Rec> recs;
  uint64_t next = 1;

  ~sn_ckpt_pool() {
    for (auto& kv : recs)
      if (kv.second.done) {
        cudaEventSynchronize(kv.second.done);
        cudaEventDestroy(kv.second.done);
      }
    if (base) cudaFree(base);
  }

  static size_t round_up(size_t x) { return (x + 255) & ~(size_t)255; }

  bool alloc(size_t bytes, size_t* off) {
    bytes = round_up(bytes ? bytes : 1);
    for (auto it = freeList.begin(); it != freeList.end(); ++it) {
      if (it->second < bytes) continue;
      *off = it->first;
      size_t rest = it->second - bytes;
      size_t restOff = it->first + bytes;
      freeList.erase(it);
      if (rest) freeList[restOff] = rest;
      used += bytes;
      return true;
    }
    return false;
  }

  void release(size_t off, size_t bytes) {
    bytes = round_up(bytes ? bytes : 1);
    used -= bytes;
    auto it = freeList.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != freeList.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      freeList.erase(nx);
    }
    if (it != freeList.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        freeList.erase(it);
      }
    }
  }

  // Reserve a record of `bytes`; the caller fills it on its stream and then
  // calls mark(handle, stream).
  bool reserve(size_t bytes, uint32_t kind, uint64_t* handle, Rec** out) {
    size_t off = 0;
    if (!alloc(bytes, &off)) {
      err = "checkpoint pool full (" + std::to_string(used) + " of " + std::to_string(cap) + " bytes in use, " +
            std::to_string(bytes) + " requested)";
      return false;
    }
    Rec r;
    r.off = off;
    r.bytes = bytes;
    r.kind = kind;
    if (cudaEventCreateWithFlags(&r.done, cudaEventDisableTiming) != cudaSuccess) {
      release(off, bytes);
      err = "cudaEventCreate failed";
      return false;
    }
    uint64_t h = next++;
    recs[h] = r;
    *handle = h;
    *out = &recs[h];
    return true;
  }

  Rec* find(uint64_t h) {
    auto it = recs.find(h);
    return it == recs.end() ? nullptr : &it->second;
  }

  bool free_rec(uint64_t h) {
    auto it = recs.find(h);
    if (it == recs.end()) {
      err = "no checkpoint " + std::to_string(h);
      return false;
    }
    if (it->second.done) {
      cudaEventSynchronize(it->second.done);
      cudaEventDestroy(it->second.done);
    }
    release(it->second.off, it->second.bytes);
    recs.erase(it);
    return true;
  }
};
