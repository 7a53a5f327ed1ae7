// vibe-model_gb300/csrc/cabi_host.cuh
//
// Call machinery of the C-ABI entry points (vibe_c_kernels.h). The reference's
// kernels promise no allocation per call and reentrancy (c_kernels.h:17-18);
// on the GPU that means:
//   * host-pointer calls: every host thread owns, per device, one
//     non-blocking stream, one pinned host staging buffer and one device
//     buffer. A call packs its inputs into the pinned buffer, moves them with
//     ONE host-to-device copy, launches, moves its outputs back with ONE copy
//     and waits for its own stream only. The buffers grow geometrically and
//     are reused, so once a thread has made a call of a given size, further
//     calls of that size allocate nothing.
//   * device-pointer (_dev) calls that need scratch: every host thread owns,
//     per device, one scratch buffer. A call orders itself after the previous
//     user of that buffer (an event recorded by the last call, waited on by
//     this call's stream), so calls on different streams never share it
//     concurrently, and a larger request frees the old buffer only after its
//     last user finished. Under stream capture the scratch is a stream-ordered
//     allocation instead (cudaMallocAsync / cudaFreeAsync, graph memory nodes).
// Every cudaMalloc / cudaMallocHost made here is counted
// (vibe_c_allocations()).
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <vector>

namespace vgb_cabi {

// A host-pointer call: declare the arrays, commit (stage inputs), launch on
// stream() with dev<T>(id), finish (copy outputs back, wait).
class HostCall {
 public:
  enum Kind { kIn = 0, kInOut = 1, kOut = 2, kScratch = 3 };
  HostCall();
  // `bytes` of host array `h`. A NULL input (kIn, kInOut) is absent: dev()
  // gives nullptr for it. A NULL kOut array stays in the staging buffer,
  // readable through host() after finish(). Returns the array's id.
  int add(const void* h, size_t bytes, Kind kind);
  bool commit();
  template <class T>
  T* dev(int id) const {
    const Arg& a = args_[id];
    if (a.absent) return nullptr;
    return reinterpret_cast<T*>(base_ + a.off);
  }
  cudaStream_t stream() const;
  bool finish();
  const void* host(int id) const;
  bool ok() const { return ok_; }

 private:
  struct Arg {
    const void* h;
    size_t bytes, off;
    Kind kind;
    bool absent;
  };
  std::vector<Arg> args_;
  void* ctx_ = nullptr;
  char* base_ = nullptr;
  size_t h2d_end_ = 0, d2h_beg_ = 0, d2h_end_ = 0;
  bool ok_ = true;
};

// Scratch of a _dev call on `stream`; release() after the launches that use
// it. Returns nullptr (and sets the thread's error) on failure.
class DevScratch {
 public:
  DevScratch(size_t bytes, cudaStream_t stream);
  ~DevScratch();
  void* get() const { return p_; }
  bool release();

 private:
  void* p_ = nullptr;
  cudaStream_t s_;
  bool graph_ = false, released_ = false;
};

void set_error(const char* what, cudaError_t e);
unsigned long long allocations();

}  // namespace vgb_cabi
