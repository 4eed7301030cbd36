// runtime.cpp — per-thread C-ABI contexts, device buffers and error mapping.
#include "usx/runtime.hpp"

#include <chrono>
#include <cstdlib>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace usx {
namespace rt {

namespace {

struct ThreadCtx {
  usx_ctx* ctx = nullptr;
  std::vector<std::unique_ptr<DeviceBuffer>> slots;
  ~ThreadCtx() {
    slots.clear();
    if (ctx) usx_cu_ctx_destroy(ctx);
  }
};

ThreadCtx& tls() {
  thread_local ThreadCtx t;
  return t;
}

}  // namespace

usx_ctx* ctx() {
  ThreadCtx& t = tls();
  if (!t.ctx) {
    int device = 0;
    if (const char* d = std::getenv("USX_DEVICE")) device = std::atoi(d);
    const int rc = usx_cu_ctx_create(device, nullptr, &t.ctx);
    if (rc != USX_OK)
      throw std::runtime_error(std::string("usx: no usable CUDA device (") + usx_cu_last_error() +
                               "); this engine has no CPU path");
  }
  return t.ctx;
}

void check(int rc, const char* what) {
  if (rc == USX_OK) return;
  const std::string msg = usx_cu_last_error();
  if (rc == USX_ERR_INVALID) throw std::invalid_argument(msg.empty() ? what : msg);
  throw std::runtime_error(std::string(what) + ": " + msg);
}

DeviceBuffer::~DeviceBuffer() {
  if (ptr_ && owner_) usx_cu_free(owner_, ptr_);
}

void* DeviceBuffer::ensure(std::size_t bytes) {
  if (bytes > bytes_) {
    usx_ctx* c = ctx();
    if (ptr_) {
      check(usx_cu_synchronize(c), "synchronize");
      usx_cu_free(c, ptr_);
      ptr_ = nullptr;
      bytes_ = 0;
    }
    const std::size_t want = bytes + bytes / 8;
    check(usx_cu_malloc(c, want, &ptr_), "device allocation");
    bytes_ = want;
    owner_ = c;
  }
  return ptr_;
}

void* slot(int index, std::size_t bytes) {
  ThreadCtx& t = tls();
  if (static_cast<int>(t.slots.size()) <= index) t.slots.resize(static_cast<std::size_t>(index) + 1);
  if (!t.slots[static_cast<std::size_t>(index)]) t.slots[static_cast<std::size_t>(index)].reset(new DeviceBuffer());
  return t.slots[static_cast<std::size_t>(index)]->ensure(bytes);
}

void h2d(void* dst, const void* src, std::size_t bytes) {
  check(usx_cu_memcpy_h2d(ctx(), dst, src, bytes), "host-to-device copy");
}
void d2h(void* dst, const void* src, std::size_t bytes) {
  check(usx_cu_memcpy_d2h(ctx(), dst, src, bytes), "device-to-host copy");
}
void sync() { check(usx_cu_synchronize(ctx()), "synchronize"); }

double now_ms() {
  using C = std::chrono::steady_clock;
  return std::chrono::duration<double, std::milli>(C::now().time_since_epoch()).count();
}

}  // namespace rt
}  // namespace usx
