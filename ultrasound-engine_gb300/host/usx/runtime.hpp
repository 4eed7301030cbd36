// usx/runtime.hpp — the host side of the device boundary: one C-ABI context
// per host thread (its own stream and scratch arena, so concurrent callers
// never share a stream), grow-only device buffers, and the mapping of C-ABI
// status codes onto the exceptions the reference throws.
#pragma once

#include <cstddef>
#include <string>

#include "usx_cu.h"

namespace usx {
namespace rt {

// The calling thread's context on the selected device (USX_DEVICE, default 0).
// Throws std::runtime_error when no CUDA device is usable: there is no CPU path.
usx_ctx* ctx();

// Throws std::invalid_argument for USX_ERR_INVALID, std::runtime_error otherwise.
void check(int rc, const char* what);

// A grow-only device allocation owned by the calling thread's context.
class DeviceBuffer {
 public:
  DeviceBuffer() = default;
  ~DeviceBuffer();
  DeviceBuffer(const DeviceBuffer&) = delete;
  DeviceBuffer& operator=(const DeviceBuffer&) = delete;
  void* ensure(std::size_t bytes);
  void* get() const { return ptr_; }

 private:
  void* ptr_ = nullptr;
  std::size_t bytes_ = 0;
  usx_ctx* owner_ = nullptr;
};

// Per-thread scratch slots for the host API's transfers (inputs, outputs).
void* slot(int index, std::size_t bytes);

void h2d(void* dst, const void* src, std::size_t bytes);
void d2h(void* dst, const void* src, std::size_t bytes);
void sync();

// Wall-clock milliseconds between two points (host steady clock).
double now_ms();

}  // namespace rt
}  // namespace usx
