// pbf_common.h -- host-side error plumbing and device buffers shared by the
// C-ABI translation units.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <array>
#include <cstddef>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "pbf103.h"

namespace pbf {

// A failure carrying the C-ABI status that maps onto the reference's
// exception type.
struct Failure : std::runtime_error {
    pbf_status status;
    Failure(pbf_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

[[noreturn]] inline void fail(pbf_status s, const std::string& m) { throw Failure(s, m); }

// Argument validation shared by the solver and the adjoint
// (PBFSolver::initialize, src/pbf/pbf_solver.cu:45-79, and SpatialGrid
// dimensions, src/pbf/spatial_grid.cu:10-64).
bool finite3(pbf_float3 v);
void validate_params(const pbf_params& p);
std::array<int, 3> grid_dims_checked(pbf_float3 mn, pbf_float3 mx, float cell);
// Validated device records of colliders (CollisionSystem setters,
// src/pbf/collision_system.cu:53-126): kind 0 spheres (center, radius), 1
// boxes (center, -), (halfExtents, -), 2 planes (point, -), (normal, -).
std::vector<float4> collider_records(int kind, const void* data, size_t count);

inline void cuda_check(cudaError_t e) {
    if (e != cudaSuccess) fail(PBF_ERR_RUNTIME, cudaGetErrorString(e));
}

// An NVTX range around one entry point, for a timeline tool (Nsight Systems)
// to show the library's calls, as the reference's benchmark marks its run and
// every physics frame (benchmark/pbf_benchmark.cu:44,125-137).  Costs a
// function-pointer check when no tool is attached.
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

// Move-only owner of one device allocation (the role CudaBuffer plays in the
// reference, include/pbf/cuda_buffer.hpp:11-139).
class DeviceBuffer {
public:
    DeviceBuffer() = default;
    explicit DeviceBuffer(size_t bytes) { allocate(bytes); }
    DeviceBuffer(const DeviceBuffer&) = delete;
    DeviceBuffer& operator=(const DeviceBuffer&) = delete;
    DeviceBuffer(DeviceBuffer&& o) noexcept
        : p_(std::exchange(o.p_, nullptr)), bytes_(std::exchange(o.bytes_, 0)) {}
    DeviceBuffer& operator=(DeviceBuffer&& o) noexcept {
        if (this != &o) {
            release();
            p_ = std::exchange(o.p_, nullptr);
            bytes_ = std::exchange(o.bytes_, 0);
        }
        return *this;
    }
    ~DeviceBuffer() { release(); }

    void allocate(size_t bytes) {
        if (bytes == 0) {
            release();
            return;
        }
        void* np = nullptr;
        cuda_check(cudaMalloc(&np, bytes));
        release();
        p_ = np;
        bytes_ = bytes;
    }
    template <class T> T* as() const { return static_cast<T*>(p_); }
    void* get() const { return p_; }
    size_t bytes() const { return bytes_; }

private:
    void release() noexcept {
        if (p_) cudaFree(p_);
        p_ = nullptr;
        bytes_ = 0;
    }
    void* p_ = nullptr;
    size_t bytes_ = 0;
};

void set_global_error(const std::string& m);

// Runs fn and converts failures into a status; msg receives the message.
template <class Fn>
pbf_status guarded(std::string* msg, Fn&& fn) {
    try {
        fn();
        if (msg) msg->clear();
        return PBF_OK;
    } catch (const Failure& f) {
        if (msg) *msg = f.what();
        set_global_error(f.what());
        return f.status;
    } catch (const std::bad_alloc&) {
        if (msg) *msg = "host allocation failed";
        set_global_error("host allocation failed");
        return PBF_ERR_RUNTIME;
    } catch (const std::exception& e) {
        if (msg) *msg = e.what();
        set_global_error(e.what());
        return PBF_ERR_RUNTIME;
    }
}

}  // namespace pbf
