// ctx.cu -- library, error and context entry points of the C ABI, the
// device Philox sampler and the FP64 re-score kernel shared by the solvers.
#include <cstring>
#include <vector>

#include "common.cuh"
#include "philox.cuh"
#include "rescore.cuh"

namespace os {

static thread_local std::string g_last_error;

os_status fail(os_status st, const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return st;
}

void throw_error(os_status st, const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  throw Error(st, buf);
}

void activate(os_ctx *ctx) {
  OS_REQUIRE(ctx != nullptr, "null context");
  OS_CUDA(cudaSetDevice(ctx->device));
}

const char *last_error_cstr() { return g_last_error.c_str(); }

// FP64 energies of m states under the reference's energy function
// (annealing.hpp:31-40): one warp per state; lane 0 walks the upper triangle
// in row-major order so the FP64 additions happen in the reference's order,
// while the other lanes stage the state's set bits. Only additions of matrix
// entries are performed (the products by 0/1 are exact), so the result is
// bit-identical to the reference's sum.
__global__ void energy_rescore_kernel(const double *__restrict__ f, int n,
                                      const uint8_t *__restrict__ states, int m,
                                      double *__restrict__ out) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (warp >= m) return;
  const uint8_t *x = states + (size_t)warp * n;
  double e = 0.0;
  if (lane == 0) e = rescore_energy(f, n, x);
  if (lane == 0) out[warp] = e;
}

void launch_rescore(const double *d_f, int n, const uint8_t *d_states, int m,
                    double *d_out, cudaStream_t stream) {
  if (m <= 0) return;
  int threads = 128;
  int blocks = (int)ceil_div_u64((uint64_t)m * 32, threads);
  energy_rescore_kernel<<<blocks, threads, 0, stream>>>(d_f, n, d_states, m, d_out);
  OS_CUDA(cudaGetLastError());
}

constexpr int RESCORE_MAX_WORDS = 64;  // n <= 2048

__global__ void __launch_bounds__(RESCORE_WARPS * 32) energy_rescore_warp_kernel(const double *__restrict__ f, int n,
                                                                                const uint8_t *__restrict__ states,
                                                                                int m, double *__restrict__ out) {
  __shared__ unsigned xw[RESCORE_MAX_WORDS];
  __shared__ double red[RESCORE_WARPS];
  const int state = blockIdx.x;
  const double e = rescore_energy_block(f, n, states + (size_t)state * n, xw, red);
  if (threadIdx.x == 0) out[state] = e;
}

void launch_rescore_warp(const double *d_f, int n, const uint8_t *d_states, int m,
                         double *d_out, cudaStream_t stream) {
  if (m <= 0) return;
  OS_REQUIRE(n <= RESCORE_MAX_WORDS * 32, "warp re-score supports up to %d variables", RESCORE_MAX_WORDS * 32);
  energy_rescore_warp_kernel<<<m, RESCORE_WARPS * 32, 0, stream>>>(d_f, n, d_states, m, d_out);
  OS_CUDA(cudaGetLastError());
}

__global__ void philox_sample_kernel(uint32_t c0, uint32_t c1, uint32_t c2,
                                     uint32_t c3, uint32_t k0, uint32_t k1,
                                     int count, uint32_t *out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  Philox4 r = philox4x32_10(c0 + (uint32_t)i, c1, c2, c3, k0, k1);
  out[4 * i + 0] = r.x;
  out[4 * i + 1] = r.y;
  out[4 * i + 2] = r.z;
  out[4 * i + 3] = r.w;
}

}  // namespace os

using namespace os;

extern "C" {

int32_t os_abi_version(void) { return OS_ABI_VERSION; }

const char *os_last_error(void) { return os::last_error_cstr(); }

const char *os_status_string(os_status status) {
  switch (status) {
    case OS_OK: return "OK";
    case OS_INVALID_ARG: return "INVALID_ARG";
    case OS_CUDA_ERROR: return "CUDA_ERROR";
    case OS_TIMEOUT: return "TIMEOUT";
    case OS_OVERFLOW_MINIMISERS: return "OVERFLOW_MINIMISERS";
    case OS_NO_DEVICE: return "NO_DEVICE";
    case OS_PARSE_ERROR: return "PARSE_ERROR";
    case OS_UNSUPPORTED: return "UNSUPPORTED";
  }
  return "UNKNOWN";
}

os_status os_select_device(const char *device_type, int32_t *device_out) {
  return guard([&] {
    OS_REQUIRE(device_type && device_out, "null argument");
    std::string t(device_type);
    if (t == "gpu") {
      int count = 0;
      cudaError_t err = cudaGetDeviceCount(&count);
      if (err != cudaSuccess || count == 0)
        throw_error(OS_NO_DEVICE, "No devices of given type could be initialized.");
      *device_out = 0;
    } else if (t == "cpu" || t == "host") {
      throw_error(OS_UNSUPPORTED,
                  "Device type %s is not available: this library runs on the GPU "
                  "only (use --device-type gpu).",
                  device_type);
    } else {
      throw_error(OS_INVALID_ARG, "Unknown device type: %s", device_type);
    }
  });
}

os_status os_device_name(int32_t device, char *buf, size_t cap) {
  return guard([&] {
    OS_REQUIRE(buf && cap > 0, "null buffer");
    cudaDeviceProp prop;
    cudaError_t err = cudaGetDeviceProperties(&prop, device);
    if (err != cudaSuccess) throw_error(OS_NO_DEVICE, "no CUDA device %d", device);
    snprintf(buf, cap, "%s", prop.name);
  });
}

os_status os_ctx_create(int32_t device, os_ctx **out) {
  return guard([&] {
    OS_REQUIRE(out != nullptr, "null output");
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count)
      throw_error(OS_NO_DEVICE, "no CUDA device %d", device);
    OS_CUDA(cudaSetDevice(device));
    auto *ctx = new os_ctx();
    ctx->device = device;
    cudaError_t err = cudaDeviceGetAttribute(&ctx->sm_count,
                                             cudaDevAttrMultiProcessorCount, device);
    if (err == cudaSuccess)
      err = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking);
    if (err == cudaSuccess) {
      cudaMemPoolProps props = {};
      props.allocType = cudaMemAllocationTypePinned;
      props.location.type = cudaMemLocationTypeDevice;
      props.location.id = device;
      err = cudaMemPoolCreate(&ctx->pool, &props);
    }
    if (err == cudaSuccess) {
      uint64_t keep = 1ull << 30;
      err = cudaMemPoolSetAttribute(ctx->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    if (err != cudaSuccess) {
      if (ctx->pool) cudaMemPoolDestroy(ctx->pool);
      if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
      delete ctx;
      throw_error(OS_CUDA_ERROR, "context creation failed: %s", cudaGetErrorString(err));
    }
    ctx->stream = ctx->own_stream;
    *out = ctx;
  });
}

os_status os_ctx_destroy(os_ctx *ctx) {
  return guard([&] {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->own_stream) {
      cudaStreamSynchronize(ctx->own_stream);
      cudaStreamDestroy(ctx->own_stream);
    }
    if (ctx->pool) cudaMemPoolDestroy(ctx->pool);
    delete ctx;
  });
}

os_status os_ctx_set_stream(os_ctx *ctx, void *stream) {
  return guard([&] {
    OS_REQUIRE(ctx != nullptr, "null context");
    ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
  });
}

os_status os_philox_sample(os_ctx *ctx, const uint32_t ctr[4], const uint32_t key[2],
                           int32_t count, uint32_t *out) {
  return guard([&] {
    activate(ctx);
    OS_REQUIRE(ctr && key && out && count > 0, "bad arguments");
    DevBuf<uint32_t> d;
    d.alloc((size_t)count * 4);
    philox_sample_kernel<<<(count + 127) / 128, 128, 0, ctx->stream>>>(
        ctr[0], ctr[1], ctr[2], ctr[3], key[0], key[1], count, d.get());
    OS_CUDA(cudaGetLastError());
    OS_CUDA(cudaMemcpyAsync(out, d.get(), sizeof(uint32_t) * 4 * count,
                            cudaMemcpyDeviceToHost, ctx->stream));
    OS_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

os_status os_energy_batch(os_ctx *ctx, const os_qubo_dense *qubo, const char *states,
                          int32_t m, double *energies) {
  return guard([&] {
    activate(ctx);
    OS_REQUIRE(qubo && qubo->f && qubo->n > 0 && states && energies && m >= 0,
               "bad arguments");
    if (m == 0) return;
    const int n = qubo->n;
    DevBuf<double> d_f, d_e;
    DevBuf<uint8_t> d_s;
    d_f.alloc((size_t)n * n);
    d_s.alloc((size_t)m * n);
    d_e.alloc(m);
    OS_CUDA(cudaMemcpyAsync(d_f.get(), qubo->f, sizeof(double) * n * n,
                            cudaMemcpyHostToDevice, ctx->stream));
    OS_CUDA(cudaMemcpyAsync(d_s.get(), states, (size_t)m * n, cudaMemcpyHostToDevice,
                            ctx->stream));
    launch_rescore(d_f.get(), n, d_s.get(), m, d_e.get(), ctx->stream);
    OS_CUDA(cudaMemcpyAsync(energies, d_e.get(), sizeof(double) * m,
                            cudaMemcpyDeviceToHost, ctx->stream));
    OS_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

}  // extern "C"
