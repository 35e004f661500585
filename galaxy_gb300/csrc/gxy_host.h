// gxy_host.h -- host-side runtime pieces shared by the translation units of
// libgxy_gpu.so: error reporting, the budgeted device arena and the scene
// object behind the gxy_scene handle.
#pragma once

#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/gxy_gpu.h"
#include "gxy_dev.cuh"

namespace gxy {

// Thread-local last error; every C entry point returns a status code.
int set_error(int code, const std::string &msg);
const std::string &last_error();

#define CK(call)                                                                                      \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess)                                                                        \
            return ::gxy::set_error(GXY_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// Device allocations counted against the HBM budget given to gxy_gpu_init.
class DeviceArena {
  public:
    int alloc(void **p, size_t bytes);
    void free(void *p);
    size_t in_use() const;
    size_t budget() const;
    void set_budget(size_t b);
    bool would_fit(size_t bytes) const;

  private:
    mutable std::mutex mu_;
    size_t in_use_ = 0, budget_ = 0;
    std::vector<std::pair<void *, size_t>> live_;
};
DeviceArena &arena();

// Frees its allocations when it goes out of scope (build temporaries).
class ScratchList {
  public:
    explicit ScratchList(DeviceArena &a) : a_(a) {}
    ~ScratchList() {
        for (void *p : ptrs_) a_.free(p);
    }
    int alloc(void **p, size_t bytes) {
        int rc = a_.alloc(p, bytes ? bytes : 16);
        if (rc == GXY_OK) ptrs_.push_back(*p);
        return rc;
    }

  private:
    DeviceArena &a_;
    std::vector<void *> ptrs_;
};

struct BVHInfo {
    unsigned n_nodes = 0, n_slots = 0;
    int levels = 0, sah_levels = 0;
    double build_ms = 0;
    void *nodes_ptr = nullptr, *slots_ptr = nullptr;
};

int build_bvh8(DevScene &S, const float *sph_radius, DeviceArena &arena, cudaStream_t st, BVHInfo &info);
// Binned-SAH top tree over radix-tree clusters of at most sah_cluster_size()
// primitives (sah_builder() true), else the radix tree alone.
bool sah_builder();
int sah_cluster_size();
// Largest subtree (primitives) stored as one leaf of a wide node, 1-4.
int leaf_max();
// Wide-node collapse by the surface-area cost programme (true) or by
// opening the largest child (false).
bool collapse_cost();

}  // namespace gxy
