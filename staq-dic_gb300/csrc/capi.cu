// C ABI of libstaqdic (declared in include/staqdic.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/staqdic.h"
#include "kernels.h"


struct stdic_ctx {
  int device = 0;
  int nsm = 0;
  cudaStream_t own = nullptr;
  cudaStream_t stream = nullptr;
  void* ws = nullptr;
  size_t ws_size = 0;
  int* scal = nullptr;  // device scalars: [1] badnum, [2] iters, [3] status, [4..5] queue heads, [6] queue split,
                        // [7] adjoint queue head, [8..9] iteration-list counts,
                        // [10] gradient tile-copy time-out flag, [12..23] plain IC-GN size-class ranges and work counters,
                        // [24..33] bad-point code statistics (5 x int64),
                        // [64..575] work-queue histogram and bin cursors
  double* scald = nullptr;  // device double scalars: [0] residual
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEvent_t es0 = nullptr, es1 = nullptr;  // around the last IC-GN solver kernel
  // side stream for host copies that overlap kernels of the same call (the
  // deformed frame's upload during the set-up stage, the Hessians' download
  // during the iterations), with the events that order it against `stream`
  cudaStream_t side = nullptr;
  cudaEvent_t evs0 = nullptr, evs1 = nullptr, evh0 = nullptr, evh1 = nullptr;
  cudaEvent_t evband[8] = {};  // end of each row band of a banded upload
  // streams and events on which the plain IC-GN size classes run concurrently
  stdic::PlainStreams plain{};
  bool solver_timed = false;
  std::string err;
  long long launches = 0;
  // autotuner cache: (N bucket, npx_max, two_dof, frames) -> index of the launch shape
  std::map<std::tuple<int, int, int, int>, int> tune;
  // resident CTAs per SM of a batched launch shape (tw, two_dof, threads,
  // tile pixels, staged floats, stage), queried from the driver once
  std::map<std::tuple<int, int, int, int, int, int>, int> occ;
  int tuning = 1;
  bool capturing = false;  // the stream is being captured into a CUDA graph
  long long wait_limit = 0;  // polls of a PCG grid-barrier wait (0: the default)
  void* aux = nullptr;       // grow-only device scratch of the mesh generation
  size_t aux_size = 0;
};

namespace {

int fail(stdic_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

int cuda_fail(stdic_ctx* c, cudaError_t e, const char* where) {
  return fail(c, STDIC_E_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

bool is_device_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// host memory the CUDA driver has pinned (cudaHostAlloc, cudaHostRegister):
// copies from and to it are asynchronous, so they can overlap kernels
bool is_pinned_host_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeHost;
}

size_t al(size_t x) { return (x + 255) & ~(size_t)255; }

// c->scal slot a kernel sets when a bounded wait for a TMA tile copy gave up
constexpr int kTmaErrSlot = 40;
// Frames of fewer than kBandMinRows rows per band are uploaded whole.
constexpr int kBandMinRows = 128;
constexpr int kBandScratch = 2 * 256 * stdic::kQueueMaxBands + 2 * stdic::kQueueMaxBands + 1;

// Plans device placement for one call: device pointers pass through, host
// buffers and scratch get regions of the context workspace.
//
// Host inputs are copied on the call's stream before its kernels, except
// "late" ones (in_late), which the side stream copies while the first kernels
// run; the call's stream waits for them (wait_late) before the first kernel
// that reads them.  Host outputs are copied after the kernels, except those
// handed to copy_early, which the side stream copies as soon as the kernels
// that write them are done, while later kernels run.  Every side-stream copy
// starts after the work the call's stream held when it was issued (so it never
// touches workspace that an earlier call still uses) and is joined back into
// the call's stream before finish() copies the rest, and in any case when the
// plan goes out of scope, so the next call on the stream is ordered after it.
// "Banded" inputs (in_banded, with set_bands) are uploaded on the side stream
// in row bands, each band's end marked by an event, so that kernels that need
// only the first rows of a frame can start (wait_band) while the rest crosses
// the host link.  A band's copies are issued when the call first waits for
// it, so that the host queues the kernels of the earlier bands in between
// (queuing one pinned copy takes the host about 13 us, and queuing every
// band up front delayed the first kernels); the late copies follow the last
// band.
// Under stream capture nothing goes to the side stream.
struct Plan {
  struct Item {
    const void* host;
    void* host_out;
    size_t bytes;
    size_t off;
    bool dev;
    int dir;  // 0 in, 1 out, 2 scratch
    void** slot;
    bool late;   // input copied on the side stream (in_late)
    bool early;  // output already copied on the side stream (copy_early)
    // banded input (in_banded): bytes per array row, rows, and the image row
    // of array row 0 (row_bytes 0: not banded)
    size_t row_bytes = 0;
    int rows = 0, row0 = 0;
  };
  int nbands = 0, band_H = 0;  // set_bands: the frame's rows in nbands bands
  bool bands_pending = false;     // banded copies in use in this call (until join)
  int bands_issued = 0;           // bands whose copies are issued
  std::vector<Item> items;
  size_t total = 0;
  bool any_host = false;
  stdic_ctx* ctx = nullptr;
  bool late_pending = false, early_pending = false, late_issued = false;

  Plan() = default;
  Plan(const Plan&) = delete;
  Plan& operator=(const Plan&) = delete;
  ~Plan() { join(); }

  template <class T>
  void in(const T* p, size_t count, T** slot) {
    Item it{p, nullptr, sizeof(T) * count, 0, is_device_ptr(p), 0, (void**)slot, false, false};
    if (!p) { *slot = nullptr; return; }
    if (!it.dev) { it.off = total; total += al(it.bytes); any_host = true; }
    items.push_back(it);
  }
  // Uploads the frame's rows in nb bands of about H / nb rows (set before
  // commit; nb <= 8).
  void set_bands(int nb, int H) {
    nbands = std::max(0, std::min(nb, 8));
    band_H = H;
  }
  // A host array of `rows` rows of `row_bytes` bytes whose row r holds image
  // row r + row0, uploaded band by band (pinned memory only; pageable memory
  // is copied in order on the call's stream).
  template <class T>
  void in_banded(const T* p, size_t count, T** slot, size_t row_bytes, int rows, int row0) {
    in(p, count, slot);
    if (p && !items.back().dev && is_pinned_host_ptr(p)) {
      items.back().row_bytes = row_bytes;
      items.back().rows = rows;
      items.back().row0 = row0;
    }
  }
  // The call's stream waits for the rows of bands 0..b (idempotent per band).
  int wait_band(int b) {
    if (!bands_pending || !ctx || b < 0 || b >= nbands) return STDIC_OK;
    const int rc = issue_bands(b);
    if (rc) return rc;
    cudaError_t e = cudaStreamWaitEvent(ctx->stream, ctx->evband[b], 0);
    return e == cudaSuccess ? STDIC_OK : cuda_fail(ctx, e, "band wait");
  }
  // Issues the copies of the bands up to b not yet issued, each followed by
  // its band's event; after the last band, the late copies and evs1.
  int issue_bands(int b) {
    if (!bands_pending || !ctx) return STDIC_OK;
    stdic_ctx* c = ctx;
    cudaError_t e = cudaSuccess;
    b = std::min(b, nbands - 1);
    for (; bands_issued <= b && e == cudaSuccess; ++bands_issued) {
      const int k = bands_issued;
      const long long beg = (long long)k * band_H / nbands, end = (long long)(k + 1) * band_H / nbands;
      for (auto& it : items) {
        if (!(it.dir == 0 && !it.dev && it.row_bytes > 0 && !it.late)) continue;
        const long long lo = std::max(0LL, std::min((long long)it.rows, beg - it.row0));
        const long long hi = k == nbands - 1 ? it.rows : std::max(0LL, std::min((long long)it.rows, end - it.row0));
        if (hi <= lo) continue;
        e = cudaMemcpyAsync((char*)*it.slot + lo * it.row_bytes, (const char*)it.host + lo * it.row_bytes,
                            (hi - lo) * it.row_bytes, cudaMemcpyHostToDevice, c->side);
        if (e != cudaSuccess) break;
      }
      if (e == cudaSuccess) e = cudaEventRecord(c->evband[k], c->side);
    }
    if (e == cudaSuccess && bands_issued == nbands && !late_issued) e = issue_late(c);
    if (e != cudaSuccess) {
      // no event marks the end of the side copies: wait for them here
      cudaStreamSynchronize(c->side);
      bands_pending = false;
      late_pending = false;
      return cuda_fail(c, e, "host-to-device copy");
    }
    return STDIC_OK;
  }
  // The late copies on the side stream, then evs1 behind them.
  cudaError_t issue_late(stdic_ctx* c) {
    cudaError_t e = cudaSuccess;
    for (auto& it : items) {
      if (!(it.dir == 0 && !it.dev && it.late)) continue;
      e = cudaMemcpyAsync(*it.slot, it.host, it.bytes, cudaMemcpyHostToDevice, c->side);
      if (e != cudaSuccess) return e;
    }
    late_issued = true;
    return cudaEventRecord(c->evs1, c->side);
  }
  // pageable host memory is copied in order on the call's stream instead
  template <class T>
  void in_late(const T* p, size_t count, T** slot) {
    in(p, count, slot);
    if (p) items.back().late = !items.back().dev && is_pinned_host_ptr(p);
  }
  template <class T>
  void out(T* p, size_t count, T** slot) {
    Item it{nullptr, p, sizeof(T) * count, 0, is_device_ptr(p), 1, (void**)slot, false, false};
    if (!p) { *slot = nullptr; return; }
    if (!it.dev) { it.off = total; total += al(it.bytes); any_host = true; }
    items.push_back(it);
  }
  template <class T>
  void scratch(size_t count, T** slot) {
    Item it{nullptr, nullptr, sizeof(T) * count, total, false, 2, (void**)slot, false, false};
    total += al(it.bytes);
    items.push_back(it);
  }
  bool copied_early(const void* const* slot) const {
    for (auto& it : items)
      if ((const void* const*)it.slot == slot) return it.early;
    return false;
  }
  // true when the output bound to slot is a host buffer that finish() would copy
  bool host_output(const void* const* slot) const {
    for (auto& it : items)
      if ((const void* const*)it.slot == slot) return it.dir == 1 && !it.dev;
    return false;
  }
  // The call's stream waits for the late inputs (idempotent), issuing the
  // bands not yet issued first.
  int wait_late() {
    const int rc = issue_bands(nbands - 1);
    if (rc) return rc;
    if (late_pending && ctx) cudaStreamWaitEvent(ctx->stream, ctx->evs1, 0);
    late_pending = false;
    return STDIC_OK;
  }
  // Copies the host output bound to slot now, on the side stream, after the
  // work the call's stream holds so far; finish() skips it.  Returns false
  // (nothing issued) when the output is not pinned host memory (a copy into
  // pageable memory would block the host until the kernels before it are
  // done) or under capture.
  bool copy_early(const void* const* slot) {
    if (!ctx || ctx->capturing || early_pending) return false;
    for (auto& it : items) {
      if ((const void* const*)it.slot != slot || it.dir != 1 || it.dev) continue;
      if (!is_pinned_host_ptr(it.host_out)) return false;
      if (cudaEventRecord(ctx->evh0, ctx->stream) != cudaSuccess ||
          cudaStreamWaitEvent(ctx->side, ctx->evh0, 0) != cudaSuccess ||
          cudaMemcpyAsync(it.host_out, *it.slot, it.bytes, cudaMemcpyDeviceToHost, ctx->side) != cudaSuccess ||
          cudaEventRecord(ctx->evh1, ctx->side) != cudaSuccess) {
        // nothing is left pending on the side stream that the call's stream
        // could miss: wait for it whole, and copy the output in finish()
        cudaGetLastError();
        cudaStreamSynchronize(ctx->side);
        return false;
      }
      it.early = true;
      early_pending = true;
      return true;
    }
    return false;
  }
  // Joins every side-stream copy into the call's stream (evs1 is recorded
  // after the last of them, banded or late).
  int join() {
    const int rc = wait_late();
    bands_pending = false;
    if (early_pending && ctx) cudaStreamWaitEvent(ctx->stream, ctx->evh1, 0);
    early_pending = false;
    return rc;
  }
  // out-or-scratch: user buffer when given, else workspace
  template <class T>
  void out_opt(T* p, size_t count, T** slot) {
    if (p) out(p, count, slot);
    else scratch(count, slot);
  }

  int commit(stdic_ctx* c) {
    if (total > c->ws_size) {
      if (c->ws) {
        cudaStreamSynchronize(c->stream);
        cudaFree(c->ws);
        c->ws = nullptr;
        c->ws_size = 0;
      }
      const size_t want = std::max(total, c->ws_size + c->ws_size / 2);
      cudaError_t e = cudaMalloc(&c->ws, want);
      if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(c, STDIC_E_NOMEM, "workspace allocation failed");
      }
      c->ws_size = want;
    }
    ctx = c;
    // Two passes: the in-order copies first, then the late ones.  A late copy
    // starts only after every in-order copy (the side stream waits for an
    // event recorded behind them), so that it overlaps the first kernels and
    // does not share the host link with the inputs those kernels wait for.
    bool any_late = false, any_banded = false;
    const bool banding = nbands > 0 && band_H > 0 && !c->capturing;
    for (auto& it : items) {
      if (it.dir == 0 && it.dev) *it.slot = const_cast<void*>(it.host);
      else if (it.dir == 1 && it.dev) *it.slot = it.host_out;
      else *it.slot = (char*)c->ws + it.off;
      if (it.dir == 0 && !it.dev) {
        if (it.late && !c->capturing) {
          any_late = true;
          continue;
        }
        if (it.row_bytes > 0 && banding) {
          any_banded = true;
          continue;
        }
        cudaError_t e = cudaMemcpyAsync(*it.slot, it.host, it.bytes, cudaMemcpyHostToDevice, c->stream);
        if (e != cudaSuccess) return cuda_fail(c, e, "host-to-device copy");
      }
    }
    if (!any_late && !any_banded) return STDIC_OK;
    cudaError_t e = cudaEventRecord(c->evs0, c->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->side, c->evs0, 0);
    if (e != cudaSuccess) return cuda_fail(c, e, "side stream");
    late_pending = true;
    late_issued = false;
    if (any_banded) {
      // band copies (and the late ones after them) are issued by wait_band
      bands_pending = true;
      bands_issued = 0;
      return STDIC_OK;
    }
    e = issue_late(c);
    if (e != cudaSuccess) {
      // no event marks the end of the side copies: wait for them here
      cudaStreamSynchronize(c->side);
      late_pending = false;
      return cuda_fail(c, e, "host-to-device copy");
    }
    return STDIC_OK;
  }

  // Copies the host outputs and synchronises the stream when any buffer of
  // the call is on the host.  A device int dev_int (a count the call
  // produced) may ride along to a host int *dst_int in the same
  // synchronisation; *delivered says whether it did.
  int finish(stdic_ctx* c, const int* dev_int = nullptr, int* dst_int = nullptr, bool* delivered = nullptr) {
    const int jrc = join();
    if (jrc) return jrc;
    if (delivered) *delivered = false;
    for (auto& it : items) {
      if (it.dir == 1 && !it.dev && !it.early) {
        cudaError_t e = cudaMemcpyAsync(it.host_out, *it.slot, it.bytes, cudaMemcpyDeviceToHost, c->stream);
        if (e != cudaSuccess) return cuda_fail(c, e, "device-to-host copy");
      }
    }
    if (any_host) {
      int terr = 0;
      cudaError_t e = cudaSuccess;
      if (dev_int && dst_int && delivered && !is_device_ptr(dst_int)) {
        e = cudaMemcpyAsync(dst_int, dev_int, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
        if (e != cudaSuccess) return cuda_fail(c, e, "scalar read-back");
        *delivered = true;
      }
      e = cudaMemcpyAsync(&terr, c->scal + kTmaErrSlot, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
      if (e != cudaSuccess) return cuda_fail(c, e, "stream synchronise");
      if (terr) {
        cudaMemsetAsync(c->scal + kTmaErrSlot, 0, sizeof(int), c->stream);
        return fail(c, STDIC_E_TIMEOUT,
                    "a bounded wait for a TMA tile copy gave up (the subsets involved were gathered from global "
                    "memory instead)");
      }
    }
    return STDIC_OK;
  }
};

// kernels: how many kernels the launcher issued
int check_launch(stdic_ctx* c, cudaError_t e, const char* what, int kernels = 1) {
  if (e != cudaSuccess) return cuda_fail(c, e, what);
  c->launches += kernels;
  return STDIC_OK;
}

// read a device int into the host (synchronises the stream)
int read_scalar(stdic_ctx* c, const int* dev, int* host) {
  cudaError_t e = cudaMemcpyAsync(host, dev, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  return e == cudaSuccess ? STDIC_OK : cuda_fail(c, e, "scalar read-back");
}

int deliver_int(stdic_ctx* c, const int* dev, int* dst) {
  if (!dst) return STDIC_OK;
  if (is_device_ptr(dst)) {
    cudaError_t e = cudaMemcpyAsync(dst, dev, sizeof(int), cudaMemcpyDeviceToDevice, c->stream);
    return e == cudaSuccess ? STDIC_OK : cuda_fail(c, e, "scalar copy");
  }
  return read_scalar(c, dev, dst);
}

}  // namespace

extern "C" {

int stdic_ctx_create(stdic_ctx** out, int device) {
  if (!out) return STDIC_E_ARG;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) {
    cudaGetLastError();
    return STDIC_E_CUDA;
  }
  stdic_ctx* c = new stdic_ctx();
  c->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, device);
  // a blocking stream: ordered with the legacy default stream, on which the
  // caller's framework usually produces and consumes device buffers
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->own, cudaStreamDefault);
  if (e == cudaSuccess) e = cudaMalloc(&c->scal, (64 + 512) * sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(c->scal, 0, (64 + 512) * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&c->scald, 8 * sizeof(double));
  if (e == cudaSuccess) e = cudaEventCreate(&c->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&c->ev1);
  if (e == cudaSuccess) e = cudaEventCreate(&c->es0);
  if (e == cudaSuccess) e = cudaEventCreate(&c->es1);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking);
  for (cudaEvent_t* ev : {&c->evs0, &c->evs1, &c->evh0, &c->evh1, &c->plain.fork, &c->plain.join[0],
                          &c->plain.join[1], &c->plain.join[2]})
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
  for (cudaEvent_t& ev : c->evband)
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
  for (cudaStream_t* st : {&c->plain.side[0], &c->plain.side[1], &c->plain.side[2]})
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(st, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    cudaGetLastError();
    delete c;
    return STDIC_E_CUDA;
  }
  c->stream = c->own;
  *out = c;
  return STDIC_OK;
}

int stdic_ctx_destroy(stdic_ctx* c) {
  if (!c) return STDIC_OK;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->ws) cudaFree(c->ws);
  if (c->aux) cudaFree(c->aux);
  if (c->scal) cudaFree(c->scal);
  if (c->scald) cudaFree(c->scald);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->es0) cudaEventDestroy(c->es0);
  if (c->es1) cudaEventDestroy(c->es1);
  for (cudaEvent_t ev : {c->evs0, c->evs1, c->evh0, c->evh1, c->plain.fork, c->plain.join[0], c->plain.join[1],
                         c->plain.join[2]})
    if (ev) cudaEventDestroy(ev);
  for (cudaEvent_t ev : c->evband)
    if (ev) cudaEventDestroy(ev);
  if (c->side) cudaStreamDestroy(c->side);
  for (cudaStream_t st : {c->plain.side[0], c->plain.side[1], c->plain.side[2]})
    if (st) cudaStreamDestroy(st);
  if (c->own) cudaStreamDestroy(c->own);
  delete c;
  return STDIC_OK;
}

int stdic_ctx_set_stream(stdic_ctx* c, void* s) {
  if (!c) return STDIC_E_ARG;
  c->stream = s ? (cudaStream_t)s : c->own;
  return STDIC_OK;
}

const char* stdic_last_error(const stdic_ctx* c) { return c ? c->err.c_str() : "null context"; }

long long stdic_kernel_launches(const stdic_ctx* c) { return c ? c->launches : 0; }

int stdic_ctx_set_wait_limit(stdic_ctx* c, long long polls) {
  if (!c || polls < 0) return STDIC_E_ARG;
  c->wait_limit = polls;
  return STDIC_OK;
}

double stdic_last_solver_ms(stdic_ctx* c) {
  if (!c || !c->solver_timed) return -1.0;
  float ms = -1.f;
  if (cudaEventSynchronize(c->es1) != cudaSuccess || cudaEventElapsedTime(&ms, c->es0, c->es1) != cudaSuccess) {
    cudaGetLastError();
    return -1.0;
  }
  return (double)ms;
}

// ---------------------------------------------------------------------------
int stdic_interp_bicubic(stdic_ctx* c, const void* F, int64_t M, int64_t N, int64_t P, const void* X,
                         const void* Y, int64_t n, void* out, int dtype) {
  if (!c) return STDIC_E_ARG;
  if (M <= 0 || N <= 0 || P <= 0 || n < 0 || (dtype != STDIC_F64 && dtype != STDIC_F32) ||
      (n > 0 && (!F || !X || !Y || !out)))
    return fail(c, STDIC_E_ARG, "ba_interp2: bad sizes or pointers");
  cudaSetDevice(c->device);
  const size_t es = dtype == STDIC_F64 ? 8 : 4;
  Plan pl;
  const unsigned char *dF, *dX, *dY;
  unsigned char* dO;
  pl.in((const unsigned char*)F, es * M * N * P, (unsigned char**)&dF);
  pl.in((const unsigned char*)X, es * n, (unsigned char**)&dX);
  pl.in((const unsigned char*)Y, es * n, (unsigned char**)&dY);
  pl.out((unsigned char*)out, es * n * P, &dO);
  int rc = pl.commit(c);
  if (rc) return rc;
  if (n > 0) {
    rc = check_launch(c, stdic::launch_interp(dF, M, N, P, dX, dY, n, dO, dtype, c->stream), "ba_interp2");
    if (rc) return rc;
  }
  return pl.finish(c);
}

int stdic_img_gradient(stdic_ctx* c, const void* img, const uint8_t* mask, int W, int H, void* dfdx,
                       void* dfdy, int dtype) {
  if (!c) return STDIC_E_ARG;
  if (W < 7 || H < 7 || !img || !mask || !dfdx || !dfdy || (dtype != STDIC_F64 && dtype != STDIC_F32))
    return fail(c, STDIC_E_ARG, "funImgGradient: image must be at least 7 x 7");
  cudaSetDevice(c->device);
  const size_t es = dtype == STDIC_F64 ? 8 : 4;
  Plan pl;
  const unsigned char* di;
  const uint8_t* dm;
  unsigned char *dx, *dy;
  pl.in((const unsigned char*)img, es * W * H, (unsigned char**)&di);
  pl.in(mask, (size_t)W * H, (uint8_t**)&dm);
  pl.out((unsigned char*)dfdx, es * (W - 6) * (H - 6), &dx);
  pl.out((unsigned char*)dfdy, es * (W - 6) * (H - 6), &dy);
  int rc = pl.commit(c);
  if (rc) return rc;
  cudaMemsetAsync(c->scal + 10, 0, sizeof(int), c->stream);
  rc = check_launch(c, stdic::launch_gradient(di, dm, W, H, dx, dy, dtype, c->stream, c->scal + 10),
                    "funImgGradient");
  if (rc) return rc;
  rc = pl.finish(c);
  if (rc || !pl.any_host) return rc;
  // the call has synchronised: report a tile copy whose bounded wait gave up
  int timed_out = 0;
  rc = read_scalar(c, c->scal + 10, &timed_out);
  if (rc) return rc;
  return timed_out ? fail(c, STDIC_E_TIMEOUT, "funImgGradient: a tile copy did not complete") : STDIC_OK;
}

// ---------------------------------------------------------------------------
static void grid_shrink(int W, int H, const int S[2], const double gridx[2], const double gridy[2],
                        const int ws[2], const int st[2], double gx[2], double gy[2], int* nx,
                        int* ny) {
  double gx0 = gridx[0], gx1 = gridx[1], gy0 = gridy[0], gy1 = gridy[1];
  while (gx0 - S[0] - 0.5 * ws[0] < 1) gx0 += 1;
  while (gy0 - S[1] - 0.5 * ws[1] < 1) gy0 += 1;
  while (gx1 + 1.5 * ws[0] + S[0] > (double)W) gx1 -= 1;
  while (gy1 + 1.5 * ws[1] + S[1] > (double)H) gy1 -= 1;
  gx[0] = gx0; gx[1] = gx1; gy[0] = gy0; gy[1] = gy1;
  *nx = (gx1 - st[0] >= gx0) ? (int)std::floor((gx1 - st[0] - gx0) / st[0]) + 1 : 0;
  *ny = (gy1 - st[1] >= gy0) ? (int)std::floor((gy1 - st[1] - gy0) / st[1]) + 1 : 0;
}

int stdic_integer_search_grid(int W, int H, const int S[2], const double gridx[2],
                              const double gridy[2], const int winsize[2], const int winstepsize[2],
                              int* nx, int* ny) {
  if (!S || !gridx || !gridy || !winsize || !winstepsize || !nx || !ny || winstepsize[0] <= 0 ||
      winstepsize[1] <= 0 || S[0] < 0 || S[1] < 0 || winsize[0] <= 0 || winsize[1] <= 0)
    return STDIC_E_ARG;
  double gx[2], gy[2];
  grid_shrink(W, H, S, gridx, gridy, winsize, winstepsize, gx, gy, nx, ny);
  return STDIC_OK;
}

int stdic_integer_search(stdic_ctx* c, const double* f, const double* g, int W, int H, const int S[2],
                         const double gridx[2], const double gridy[2], const int winsize[2],
                         const int winstepsize[2], double* x, double* y, double* u, double* v,
                         double* cc, int32_t* peak_rc, double* qfactors) {
  if (!c) return STDIC_E_ARG;
  int nx, ny;
  if (stdic_integer_search_grid(W, H, S, gridx, gridy, winsize, winstepsize, &nx, &ny) ||
      !f || !g || !x || !y || !u || !v || !cc)
    return fail(c, STDIC_E_ARG, "funIntegerSearch: bad arguments");
  double gx[2], gy[2];
  grid_shrink(W, H, S, gridx, gridy, winsize, winstepsize, gx, gy, &nx, &ny);
  cudaSetDevice(c->device);
  const size_t npt = (size_t)nx * ny;
  Plan pl;
  const double *df, *dg;
  double *dx, *dy, *du, *dv, *dc;
  int32_t* dp;
  pl.in(f, (size_t)W * H, (double**)&df);
  pl.in(g, (size_t)W * H, (double**)&dg);
  pl.out(x, npt, &dx); pl.out(y, npt, &dy); pl.out(u, npt, &du); pl.out(v, npt, &dv);
  pl.out(cc, npt, &dc);
  pl.out(peak_rc, 2 * npt, &dp);
  double *dq = nullptr, *qscr = nullptr;
  if (qfactors) {
    pl.out(qfactors, 2 * npt, &dq);
    pl.scratch(stdic::intsearch_qfactor_scratch_bytes(nx, ny, S[0], S[1], winsize[0], winsize[1]) / sizeof(double),
               &qscr);
  }
  int rc = pl.commit(c);
  if (rc) return rc;
  if (npt > 0) {
    rc = check_launch(c, stdic::launch_intsearch(df, dg, W, H, S[0], S[1], gx[0], gy[0], nx, ny, winsize[0],
                                                 winsize[1], winstepsize[0], winstepsize[1], dx, dy, du,
                                                 dv, dc, dp, c->stream),
                      "funIntegerSearch");
    if (rc) return rc;
    if (qfactors) {
      rc = check_launch(c, stdic::launch_intsearch_qfactors(df, dg, W, S[0], S[1], gx[0], gy[0], nx, ny, winsize[0],
                                                            winsize[1], winstepsize[0], winstepsize[1], qscr, dq,
                                                            c->stream),
                        "funIntegerSearch quality factors", 2);
      if (rc) return rc;
    }
  }
  return pl.finish(c);
}

// ---------------------------------------------------------------------------
// IC-GN drivers
// ---------------------------------------------------------------------------
namespace {

struct FrameDev {
  const void *f, *g, *dfdx, *dfdy;
  const uint8_t* mask;
  const float *f32, *g32, *dfdx32, *dfdy32;
};

// late_g: a host deformed frame is uploaded on the side stream (Plan::in_late)
// while the first kernels run; the caller waits for it before reading g.
// banded: the reference frame, its gradients and the mask are uploaded in row
// bands (Plan::in_banded; the gradient arrays' row r is image row r + 3).
int stage_frame(stdic_ctx* c, Plan& pl, const stdic_frame* fr, FrameDev* d, bool want_f32,
                int frames, bool late_g = false, bool banded = false) {
  const size_t es = fr->dtype == STDIC_F64 ? 8 : 4;
  const size_t np = (size_t)fr->W * fr->H, ng = (size_t)(fr->W - 6) * (fr->H - 6);
  const int W = fr->W, H = fr->H;
  if (banded) pl.in_banded((const unsigned char*)fr->f, es * np, (unsigned char**)&d->f, es * W, H, 0);
  else pl.in((const unsigned char*)fr->f, es * np, (unsigned char**)&d->f);
  if (late_g) pl.in_late((const unsigned char*)fr->g, es * np * frames, (unsigned char**)&d->g);
  else pl.in((const unsigned char*)fr->g, es * np * frames, (unsigned char**)&d->g);
  if (banded) {
    pl.in_banded((const unsigned char*)fr->dfdx, es * ng, (unsigned char**)&d->dfdx, es * (W - 6), H - 6, 3);
    pl.in_banded((const unsigned char*)fr->dfdy, es * ng, (unsigned char**)&d->dfdy, es * (W - 6), H - 6, 3);
    pl.in_banded(fr->mask, np, (uint8_t**)&d->mask, (size_t)W, H, 0);
  } else {
    pl.in((const unsigned char*)fr->dfdx, es * ng, (unsigned char**)&d->dfdx);
    pl.in((const unsigned char*)fr->dfdy, es * ng, (unsigned char**)&d->dfdy);
    pl.in(fr->mask, np, (uint8_t**)&d->mask);
  }
  d->f32 = d->g32 = d->dfdx32 = d->dfdy32 = nullptr;
  if (want_f32 && fr->dtype == STDIC_F64) {
    pl.scratch(np, (float**)&d->f32);
    pl.scratch(np * frames, (float**)&d->g32);
    pl.scratch(ng, (float**)&d->dfdx32);
    pl.scratch(ng, (float**)&d->dfdy32);
  }
  (void)c;
  return STDIC_OK;
}

int convert_frame(stdic_ctx* c, const stdic_frame* fr, FrameDev* d, int frames) {
  if (fr->dtype == STDIC_F32) {
    d->f32 = (const float*)d->f; d->g32 = (const float*)d->g;
    d->dfdx32 = (const float*)d->dfdx; d->dfdy32 = (const float*)d->dfdy;
    return STDIC_OK;
  }
  const long long np = (long long)fr->W * fr->H, ng = (long long)(fr->W - 6) * (fr->H - 6);
  int rc = check_launch(c, stdic::launch_to_f32((const double*)d->f, (float*)d->f32, np, c->stream), "to_f32");
  if (!rc) rc = check_launch(c, stdic::launch_to_f32((const double*)d->g, (float*)d->g32, np * frames, c->stream), "to_f32");
  if (!rc) rc = check_launch(c, stdic::launch_to_f32((const double*)d->dfdx, (float*)d->dfdx32, ng, c->stream), "to_f32");
  if (!rc) rc = check_launch(c, stdic::launch_to_f32((const double*)d->dfdy, (float*)d->dfdy32, ng, c->stream), "to_f32");
  return rc;
}

bool frame_ok(const stdic_frame* fr) {
  return fr && fr->f && fr->g && fr->mask && fr->dfdx && fr->dfdy && fr->W >= 7 && fr->H >= 7 &&
         (fr->dtype == STDIC_F64 || fr->dtype == STDIC_F32);
}

// Candidate launch shapes of the persistent batched kernel: (warps per
// subset, threads per CTA), each with its resident grid, its shared tile slot
// and the global scratch its teams need.
// split > 0: subsets of at least `split` pixels a side run on teams of tw
// warps, the rest on single warps (queue in decreasing size).
struct BatchedCand {
  int tw, threads, split, smem_per_warp, gtile_per_warp, blocks, smem_px, smem_px_small;
  int blocks1;  // grid of the 6-DOF set-up stage (fewer registers, more resident CTAs)
  size_t scratch;
};

std::vector<BatchedCand> batched_candidates(stdic_ctx* c, bool two, int npx_max, int Ntot) {
  std::vector<BatchedCand> out;
  // (warps per team, threads, split size, shared bytes per warp for the
  // per-pixel arrays, floats per warp for the staged g footprint).  A smaller
  // per-pixel slot leaves more of the SM's unified L1 to cache the gradients;
  // tiles that do not fit use the warp's global slice, footprints that do not
  // fit are gathered from global memory.
  const int shapes[][5] = {{1, 256, 0, 12800, 0},   {4, 256, 64, 5600, 0},
                           {1, 256, 0, 5600, 1600}, {1, 256, 0, 9600, 1600},
                           {4, 256, 32, 5600, 1300}, {4, 256, 64, 5600, 1300},
                           {8, 256, 64, 5600, 650},  {4, 256, 32, 5600, 1600},
                           {2, 256, 32, 5600, 1300}, {1, 256, 0, 5600, 0},
                           {2, 256, 64, 5600, 0},    {4, 256, 32, 5600, 0},
                           {2, 256, 32, 5600, 0}};
  for (auto& sh : shapes) {
    const int tw = sh[0], threads = sh[1], split = sh[2], per_warp = sh[3], gt_warp = sh[4];
    const int teams_per_block = threads / (32 * tw);
    const int bpp = stdic::batched_tile_px_bytes(two);
    int smem_px = (int)((per_warp * tw - 512 - 32 * 4 * tw) / bpp);
    smem_px = std::max(64, std::min(smem_px, npx_max));
    const int gtile = gt_warp * tw;
    auto occupancy = [&](int stage) {
      const auto key = std::make_tuple(tw, (int)two, threads, smem_px, gtile, stage);
      auto hit = c->occ.find(key);
      if (hit != c->occ.end()) return hit->second;
      const int n = stdic::batched_blocks_per_sm(tw, two, threads, smem_px, gtile, stage);
      c->occ.emplace(key, n);
      return n;
    };
    const int per_sm = occupancy(2);
    if (per_sm <= 0) continue;
    const int per_sm1 = two ? per_sm : std::max(per_sm, occupancy(1));
    const int units_per_block = split ? threads / 32 : teams_per_block;
    const int max_blocks = (Ntot + units_per_block - 1) / units_per_block;
    const int blocks = std::max(1, std::min(c->nsm * per_sm, max_blocks));
    const int blocks1 = std::max(1, std::min(c->nsm * per_sm1, max_blocks));
    // global scratch slices for every warp of the larger of the two grids
    const long long warps = (long long)std::max(blocks, blocks1) * (threads / 32);
    const int small_px = split ? stdic::batched_small_px(smem_px, two, tw, gtile) : 0;
    out.push_back({tw, threads, split, per_warp, gt_warp, blocks, smem_px, small_px, blocks1,
                   stdic::batched_scratch_bytes(npx_max, two, warps)});
  }
  return out;
}

size_t batched_scratch_need(const std::vector<BatchedCand>& cs) {
  size_t m = 256;
  for (auto& cd : cs) m = std::max(m, cd.scratch);
  return m;
}

// Run the persistent batched kernel with the autotuned launch shape.  On a new
// problem class every candidate is timed once on the real data (the outputs
// are idempotent) and the fastest is cached in the context.
// STDIC_TUNE_LOG=1 prints the autotuner's timing of every candidate to stderr.
bool tune_log() {
  static const bool on = [] {
    const char* e = std::getenv("STDIC_TUNE_LOG");
    return e && e[0] == '1';
  }();
  return on;
}

// STDIC_TUNE_PICK=<k> takes launch shape k of batched_candidates without
// timing the others (for profiling one fixed configuration).
int tune_pick() {
  static const int k = [] {
    const char* e = std::getenv("STDIC_TUNE_PICK");
    return e && *e ? std::atoi(e) : -1;
  }();
  return k;
}

// STDIC_UPLOAD_BANDS=<n> (0, 1, 2, 4 or 8, default 4; other values round
// down): row bands of a host reference frame in pinned memory (0: upload it
// whole before the set-up stage).
int upload_bands() {
  static const int n = [] {
    const char* e = std::getenv("STDIC_UPLOAD_BANDS");
    const int v = e && *e ? std::max(0, std::min(8, std::atoi(e))) : 4;
    return v >= 8 ? 8 : v >= 4 ? 4 : v >= 2 ? 2 : v;
  }();
  return n;
}

// Subset sizes the work queue is sorted by (one of ws_list, wsl2, ws_all).
struct QueueKeys {
  const int32_t* ws_list;
  const int32_t* wsl2;
  int ws_all;
};

// Row bands of a frame uploaded band by band (Plan::in_banded): nb bands of
// an H-row frame, with kBandScratch ints of device scratch for the banded
// queue (its histogram and cursors, then each band's first position and
// wide-team count).
struct Bands {
  int nb = 0, H = 0;
  int32_t* buf = nullptr;
};

// pl (optional): the call's plan; the iteration stage waits for its late
// inputs, and early_slot names an output (the Hessians) that the set-up stage
// completes and that the side stream copies to the host during the iterations
// of the final launch.  bands (optional, 6-DOF, one frame): when the plan
// uploads the frame in row bands, the final launch runs the set-up stage band
// by band, each part as soon as its rows are on the device.
int run_batched(stdic_ctx* c, stdic::BatchedArgs& b, int Ntot, const std::vector<BatchedCand>& cands,
                const QueueKeys& qk, Plan* pl = nullptr, const void* const* early_slot = nullptr,
                const Bands* bands = nullptr) {
  const bool two = b.two_dof != 0;
  if (cands.empty()) return fail(c, STDIC_E_UNSUPPORTED, "no launch shape fits this subset size");
  b.queue_head = c->scal + 4;  // [4] team phase, [5] single-warp phase
  b.n_big = c->scal + 6;
  // tensor maps of the deformed frame(s) for the TMA footprint copies
  b.gbox_n = 0;
  b.tma_err = c->scal + kTmaErrSlot;
  {
    const int nf = b.frames > 0 ? b.frames : 1;
    const bool stacked_ok = nf == 1 || b.g_stride == (long long)b.a.W * b.a.H;
    if (b.g32 && stacked_ok) {
      int n = 0;
      while (n < stdic::kGBoxes && stdic::encode_image_map_f32(b.g32, b.a.W, (long long)b.a.H * nf, stdic::gbox_side(n),
                                                               &b.gmap[n]))
        ++n;
      b.gbox_n = n == stdic::kGBoxes ? n : 0;
    }
  }
  auto launch = [&](const BatchedCand& cd, bool final) -> int {
    b.warps_per_subset = cd.tw;
    b.smem_px = cd.smem_px;
    b.split = cd.split > 0 ? 1 : 0;
    b.smem_px_small = cd.smem_px_small;
    b.gtile = cd.gtile_per_warp * cd.tw;
    b.gtile_small = cd.split ? cd.gtile_per_warp : 0;
    // Single warps take the queue smallest first, so that the small subsets
    // that run to the iteration limit start early.  The split form takes it
    // largest first: its wide teams already start with the masked subsets
    // (the long chains) in the 6-DOF iteration stage, and the single-warp
    // list, filled in set-up order, then runs largest first too.
    const int mode = cd.split ? (two ? 2 : 0) : (cd.tw == 1 ? 1 : 0);
    // set-up by row band (final launch of a frame uploaded in bands): the
    // queue grouped by band, then one set-up launch per band, each after its
    // band's copies
    const bool banded = final && !two && b.frames <= 1 && !qk.wsl2 && bands && bands->nb > 0 && pl &&
                        pl->bands_pending;
    int* boff = banded ? bands->buf + 2 * 256 * stdic::kQueueMaxBands : nullptr;
    int rc = check_launch(c, banded ? stdic::launch_build_band_queue(qk.ws_list, qk.ws_all, b.a.N, b.a.coords + b.a.N,
                                                                     bands->H, bands->nb, (int32_t*)b.order,
                                                                     c->scal + 6, boff, boff + bands->nb + 1,
                                                                     bands->buf, c->stream, mode, cd.split)
                                    : stdic::launch_build_queue(qk.ws_list, qk.wsl2, qk.ws_all, b.a.N,
                                                                (int32_t*)b.order, c->scal + 6, c->scal + 64,
                                                                c->stream, mode, cd.split),
                          "queue", 3);
    if (rc) return rc;
    // 2-DOF: one fused pass; 6-DOF: set-up, FP64 factorisation, iterations
    const int stages[2] = {two ? 0 : 1, 2};
    b.split_ws = cd.split;
    b.n2 = c->scal + 8;
    if (!two) {
      cudaError_t e = cudaMemsetAsync(b.n2, 0, 2 * sizeof(int), c->stream);
      if (e != cudaSuccess) return cuda_fail(c, e, "list reset");
    }
    if (banded) {
      b.stage = 1;
      for (int k = 0; k < bands->nb; ++k) {
        rc = pl->wait_band(k);
        if (rc) return rc;
        cudaError_t e = cudaMemsetAsync(b.queue_head, 0, 2 * sizeof(int), c->stream);
        if (e != cudaSuccess) return cuda_fail(c, e, "queue reset");
        b.band_list = (const int32_t*)b.order;
        b.band_off = boff;
        b.band_nbig = boff + bands->nb + 1;
        b.band = k;
        rc = check_launch(c, stdic::launch_icgn_batched(b, cd.blocks1, cd.threads, c->stream), "IC-GN batched");
        b.band_list = nullptr;
        b.band_off = b.band_nbig = nullptr;
        b.band = 0;
        if (rc) return rc;
      }
    } else if (pl) {
      rc = pl->wait_band(pl->nbands - 1);  // the whole frame (no-op when not banded)
      if (rc) return rc;
    }
    for (int k = 0; k < (two ? 1 : 2); ++k) {
      b.stage = stages[k];
      if (!(banded && b.stage == 1)) {
        cudaError_t e = cudaMemsetAsync(b.queue_head, 0, 2 * sizeof(int), c->stream);
        if (e != cudaSuccess) return cuda_fail(c, e, "queue reset");
        // the deformed frame is read from the iteration stage on (the fused
        // 2-DOF pass reads it throughout)
        if (pl && b.stage != 1) rc = pl->wait_late();
        if (rc) return rc;
        rc = check_launch(c, stdic::launch_icgn_batched(b, b.stage == 1 ? cd.blocks1 : cd.blocks, cd.threads, c->stream),
                          "IC-GN batched");
        if (rc) return rc;
      }
      if (!two && k == 0) {
        rc = check_launch(c, stdic::launch_factor6((const stdic::SubsetState6*)b.st6, b.H6, b.Hinv6, Ntot,
                                                   b.order2, b.order2 ? b.n2 : nullptr, c->stream),
                          "Hessian factorisation");
        if (rc) return rc;
        if (final && pl && early_slot) pl->copy_early(early_slot);
      }
    }
    return STDIC_OK;
  };
  const int nb = Ntot <= 0 ? 0 : (int)std::ceil(std::log2((double)Ntot));
  const auto key = std::make_tuple(nb, b.a.npx_max, (int)two, b.frames);
  auto it = c->tune.find(key);
  if (it == c->tune.end() && c->capturing) {
    // no timing inside a capture: the first shape (or the fixed one) for this
    // launch only, not cached, so the next uncaptured call still tunes
    const int pick = tune_pick();
    return launch(cands[pick >= 0 ? std::min(pick, (int)cands.size() - 1) : 0], true);
  }
  if (it == c->tune.end()) {
    int best = 0;
    const int pick = tune_pick();
    if (pick >= 0) {
      best = std::min(pick, (int)cands.size() - 1);
    } else if (c->tuning && Ntot > 0 && cands.size() > 1) {
      float bt = 1e30f;
      for (auto& cd : cands) {
        cudaEventRecord(c->ev0, c->stream);
        const int rc = launch(cd, false);
        cudaEventRecord(c->ev1, c->stream);
        if (rc) return rc;
        cudaEventSynchronize(c->ev1);
        float ms = 0;
        cudaEventElapsedTime(&ms, c->ev0, c->ev1);
        if (ms < bt) { bt = ms; best = (int)(&cd - cands.data()); }
        if (tune_log())
          std::fprintf(stderr, "stdic tune: N=%d two=%d warps/team=%d threads=%d split=%d smem/warp=%d gtile/warp=%d blocks=%d smem_px=%d: %.3f ms\n",
                       Ntot, (int)two, cd.tw, cd.threads, cd.split, cd.smem_per_warp, cd.gtile_per_warp, cd.blocks, cd.smem_px, ms);
      }
    }
    it = c->tune.emplace(key, best).first;
  }
  const BatchedCand* chosen = &cands[std::min<size_t>((size_t)it->second, cands.size() - 1)];
  if (c->capturing) return launch(*chosen, true);
  cudaEventRecord(c->es0, c->stream);
  const int rc = launch(*chosen, true);
  cudaEventRecord(c->es1, c->stream);
  c->solver_timed = rc == STDIC_OK;
  return rc;
}

}  // namespace

static int icgn_local_impl(stdic_ctx* c, const stdic_frame* fr, const double* U0, const double* coords,
                           int N, int winsize, const int32_t* ws_list, double tol, double* U, double* F,
                           double* Hpk, int32_t* conv, uint8_t* mark_hole, int* badnum, int precision,
                           bool filter, int frames = 1) {
  if (!c) return STDIC_E_ARG;
  if (frames < 1 || (frames > 1 && (precision != STDIC_BATCHED_F32 || filter)))
    return fail(c, STDIC_E_ARG, "several frames: batched precision only, frames >= 1");
  const size_t NT = (size_t)N * frames;
  if (N < 0 || !frame_ok(fr) || (N > 0 && (!U0 || !coords || !U)) || winsize <= 0 || (winsize & 1) ||
      winsize > 96 || !(tol > 0))
    return fail(c, STDIC_E_ARG, "LocalICGNQuadtree: bad arguments (winsize even, 2..96)");
  if (precision == STDIC_PLAIN_F64 && fr->dtype != STDIC_F64)
    return fail(c, STDIC_E_ARG, "plain FP64 IC-GN needs double images");
  if (precision != STDIC_PLAIN_F64 && precision != STDIC_BATCHED_F32)
    return fail(c, STDIC_E_ARG, "unknown precision");
  cudaSetDevice(c->device);
  const bool batched = precision == STDIC_BATCHED_F32;
  Plan pl;
  FrameDev d;
  // batched FP32 frames: g is first read by the iteration stage, so a host
  // g is uploaded while the queue, set-up and factorisation kernels run; one
  // frame: the rest of the frame is uploaded in row bands, each band's
  // set-up starting as soon as its rows are on the device
  const bool f32b = batched && fr->dtype == STDIC_F32;
  Bands bands;
  if (f32b && frames == 1 && N > 0 && upload_bands() > 0 && fr->H >= upload_bands() * kBandMinRows)
    bands.nb = upload_bands(), bands.H = fr->H;
  stage_frame(c, pl, fr, &d, batched, frames, f32b, bands.nb > 0);
  pl.set_bands(bands.nb, bands.H);
  stdic::IcgnArgs a{};
  pl.in(U0, 2 * NT, (double**)&a.U0);
  pl.in(coords, 2 * (size_t)N, (double**)&a.coords);
  pl.in(ws_list, (size_t)N, (int32_t**)&a.ws_list);
  pl.out(U, 2 * NT, &a.U);
  pl.out_opt(F, 4 * NT, &a.F);
  pl.out(Hpk, 21 * NT, &a.Hpk);
  pl.out_opt(conv, NT, &a.conv);
  pl.out(mark_hole, NT, &a.mark);
  int32_t* order = nullptr;
  unsigned char* bscr = nullptr;
  const int npx_max = stdic::grown_tile_pixels(winsize);
  std::vector<BatchedCand> cands;
  stdic::SubsetState6* st6 = nullptr;
  double *H6 = nullptr, *Hinv6 = nullptr;
  int32_t* order2 = nullptr;
  pl.scratch((size_t)std::max(N, 1), &order);
  if (batched) {
    const size_t nt = std::max(NT, (size_t)1);
    cands = batched_candidates(c, false, npx_max, (int)NT);
    pl.scratch(batched_scratch_need(cands), &bscr);
    pl.scratch(nt, &st6);
    pl.scratch(21 * nt, &H6);
    pl.scratch(36 * nt, &Hinv6);
    pl.scratch(2 * nt, &order2);
    if (bands.nb > 0) pl.scratch((size_t)kBandScratch, &bands.buf);
  }
  int rc = pl.commit(c);
  if (rc) return rc;
  a.f = d.f; a.g = d.g; a.mask = d.mask; a.dfdx = d.dfdx; a.dfdy = d.dfdy;
  a.W = fr->W; a.H = fr->H; a.N = N;
  a.ws_all = winsize; a.ws_max = winsize; a.tol = tol;
  a.npx_max = npx_max;
  bool early_h = false;  // HtempPar copied to the host during the iterations
  if (N > 0) {
    if (!batched) {
      pl.wait_late();
      cudaEventRecord(c->es0, c->stream);
      int nk = 0;
      rc = check_launch(c, stdic::launch_icgn6_plain(a, order, c->scal + 64, c->scal + 12, c->stream, &nk, &c->plain),
                        "IC-GN plain", 0);
      c->launches += nk;
      cudaEventRecord(c->es1, c->stream);
      c->solver_timed = rc == STDIC_OK;
    } else {
      rc = convert_frame(c, fr, &d, frames);
      if (!rc) {
        stdic::BatchedArgs b{};
        b.a = a;
        b.f32 = d.f32; b.g32 = d.g32; b.dfdx32 = d.dfdx32; b.dfdy32 = d.dfdy32;
        b.order = order; b.two_dof = 0; b.frames = frames;
        b.g_stride = (long long)fr->W * fr->H;
        b.scratch = bscr;
        b.st6 = st6; b.H6 = H6; b.Hinv6 = Hinv6; b.order2 = order2;
        // host HtempPar with host result codes: the set-up stage writes every
        // row the iterations keep, so the rows are copied to the host during
        // the iterations; the iteration stage only zeroes the rows of the
        // subsets it ends with a run-time error (code -1), which the host
        // then zeroes in its copy from the codes
        early_h = pl.host_output((const void* const*)&a.Hpk) && pl.host_output((const void* const*)&a.conv);
        rc = run_batched(c, b, (int)NT, cands, QueueKeys{a.ws_list, nullptr, winsize}, &pl,
                         early_h ? (const void* const*)&a.Hpk : nullptr, &bands);
        early_h = early_h && pl.copied_early((const void* const*)&a.Hpk);
      }
    }
    if (rc) return rc;
    if (filter) {
      rc = check_launch(c, stdic::launch_badpoints(a.conv, N, a.U, a.F, 0, c->scal + 1, (unsigned long long*)(c->scal + 24), c->stream), "bad points", 2);
      if (rc) return rc;
    }
  } else if (filter) {
    cudaMemsetAsync(c->scal + 1, 0, sizeof(int), c->stream);
  }
  bool delivered = false;
  rc = pl.finish(c, filter ? c->scal + 1 : nullptr, filter ? badnum : nullptr, &delivered);
  if (rc) return rc;
  if (early_h) {
    for (size_t k = 0; k < NT; ++k)
      if (conv[k] == -1)
        for (int q = 0; q < 21; ++q) Hpk[(size_t)q * NT + k] = 0.0;
  }
  return filter && !delivered ? deliver_int(c, c->scal + 1, badnum) : STDIC_OK;
}

int stdic_icgn_local(stdic_ctx* c, const stdic_frame* fr, const double* U0, const double* coords, int N,
                     int winsize, const int32_t* ws_list, double tol, double* U, double* F, double* Hpk,
                     int32_t* conv, uint8_t* mark_hole, int* badnum, int precision) {
  return icgn_local_impl(c, fr, U0, coords, N, winsize, ws_list, tol, U, F, Hpk, conv, mark_hole, badnum,
                         precision, true);
}

int stdic_icgn_subsets(stdic_ctx* c, const stdic_frame* fr, const double* U0, const double* coords, int N,
                       int winsize, const int32_t* ws_list, double tol, double* U, double* F, double* Hpk,
                       int32_t* conv, int precision) {
  return icgn_local_impl(c, fr, U0, coords, N, winsize, ws_list, tol, U, F, Hpk, conv, nullptr, nullptr,
                         precision, false);
}

int stdic_icgn_subsets_frames(stdic_ctx* c, const stdic_frame* fr, int frames, const double* U0,
                              const double* coords, int N, int winsize, const int32_t* ws_list, double tol,
                              double* U, double* F, double* Hpk, int32_t* conv, int precision) {
  return icgn_local_impl(c, fr, U0, coords, N, winsize, ws_list, tol, U, F, Hpk, conv, nullptr, nullptr,
                         precision, false, frames);
}

static int subpb1_impl(stdic_ctx* c, const stdic_frame* fr, const double* UOld, const double* FOld,
                       const double* udual, const double* vdual, const double* coords, int N,
                       const int32_t* winsize_list, double mu, double beta, double tol, double* U,
                       int32_t* conv, int* badnum, int precision, bool filter);

int stdic_subpb1(stdic_ctx* c, const stdic_frame* fr, const double* UOld, const double* FOld,
                 const double* udual, const double* vdual, const double* coords, int N,
                 const int32_t* winsize_list, double mu, double beta, double tol, double* U, int32_t* conv,
                 int* badnum, int precision) {
  return subpb1_impl(c, fr, UOld, FOld, udual, vdual, coords, N, winsize_list, mu, beta, tol, U, conv,
                     badnum, precision, true);
}

int stdic_subpb1_subsets(stdic_ctx* c, const stdic_frame* fr, const double* UOld, const double* FOld,
                         const double* vdual, const double* coords, int N, const int32_t* winsize_list,
                         double mu, double tol, double* U, int32_t* conv, int precision) {
  return subpb1_impl(c, fr, UOld, FOld, nullptr, vdual, coords, N, winsize_list, mu, 0.0, tol, U, conv,
                     nullptr, precision, false);
}

static int subpb1_impl(stdic_ctx* c, const stdic_frame* fr, const double* UOld, const double* FOld,
                       const double* udual, const double* vdual, const double* coords, int N,
                       const int32_t* winsize_list, double mu, double beta, double tol, double* U,
                       int32_t* conv, int* badnum, int precision, bool filter) {
  (void)udual;
  (void)beta;
  if (!c) return STDIC_E_ARG;
  if (N < 0 || !frame_ok(fr) || (N > 0 && (!UOld || !FOld || !vdual || !coords || !winsize_list || !U)) ||
      !(tol > 0))
    return fail(c, STDIC_E_ARG, "Subpb1Quadtree: bad arguments");
  if (precision == STDIC_PLAIN_F64 && fr->dtype != STDIC_F64)
    return fail(c, STDIC_E_ARG, "plain FP64 IC-GN needs double images");
  if (precision != STDIC_PLAIN_F64 && precision != STDIC_BATCHED_F32)
    return fail(c, STDIC_E_ARG, "unknown precision");
  cudaSetDevice(c->device);
  const bool batched = precision == STDIC_BATCHED_F32;
  // the largest tile follows from the largest requested subset edge
  int wmax = 2;
  {
    std::vector<int32_t> wl(2 * (size_t)N);
    if (N > 0) {
      if (is_device_ptr(winsize_list)) {
        cudaMemcpyAsync(wl.data(), winsize_list, wl.size() * 4, cudaMemcpyDeviceToHost, c->stream);
        cudaStreamSynchronize(c->stream);
      } else {
        std::memcpy(wl.data(), winsize_list, wl.size() * 4);
      }
    }
    for (int32_t w : wl) wmax = std::max(wmax, (int)w);
  }
  if (wmax > 96) return fail(c, STDIC_E_ARG, "Subpb1Quadtree: winsize_List entries must be <= 96");
  Plan pl;
  FrameDev d;
  stage_frame(c, pl, fr, &d, batched, 1);
  stdic::IcgnArgs a{};
  pl.in(UOld, 2 * (size_t)N, (double**)&a.UOld);
  pl.in(FOld, 4 * (size_t)N, (double**)&a.FOld);
  pl.in(vdual, 2 * (size_t)N, (double**)&a.vdual);
  pl.in(coords, 2 * (size_t)N, (double**)&a.coords);
  pl.in(winsize_list, 2 * (size_t)N, (int32_t**)&a.wsl2);
  pl.out(U, 2 * (size_t)N, &a.U);
  pl.out_opt(conv, (size_t)N, &a.conv);
  int32_t* order = nullptr;
  unsigned char* bscr = nullptr;
  const int npx_max = stdic::grown_tile_pixels(wmax);
  std::vector<BatchedCand> cands;
  pl.scratch((size_t)std::max(N, 1), &order);
  if (batched) {
    cands = batched_candidates(c, true, npx_max, N);
    pl.scratch(batched_scratch_need(cands), &bscr);
  }
  int rc = pl.commit(c);
  if (rc) return rc;
  a.f = d.f; a.g = d.g; a.mask = d.mask; a.dfdx = d.dfdx; a.dfdy = d.dfdy;
  a.W = fr->W; a.H = fr->H; a.N = N; a.mu = mu; a.tol = tol; a.ws_max = wmax;
  a.npx_max = npx_max;
  if (N > 0) {
    if (!batched) {
      cudaEventRecord(c->es0, c->stream);
      int nk = 0;
      rc = check_launch(c, stdic::launch_icgn2_plain(a, order, c->scal + 64, c->scal + 12, c->stream, &nk, &c->plain),
                        "Subpb1 plain", 0);
      c->launches += nk;
      cudaEventRecord(c->es1, c->stream);
      c->solver_timed = rc == STDIC_OK;
    } else {
      rc = convert_frame(c, fr, &d, 1);
      if (!rc) {
        stdic::BatchedArgs b{};
        b.a = a;
        b.f32 = d.f32; b.g32 = d.g32; b.dfdx32 = d.dfdx32; b.dfdy32 = d.dfdy32;
        b.order = order; b.two_dof = 1; b.frames = 1; b.g_stride = 0;
        b.scratch = bscr;
        rc = run_batched(c, b, N, cands, QueueKeys{nullptr, a.wsl2, 0});
      }
    }
    if (rc) return rc;
    if (filter) {
      rc = check_launch(c, stdic::launch_badpoints(a.conv, N, a.U, nullptr, 1, c->scal + 1, (unsigned long long*)(c->scal + 24), c->stream), "bad points", 2);
      if (rc) return rc;
    }
  } else if (filter) {
    cudaMemsetAsync(c->scal + 1, 0, sizeof(int), c->stream);
  }
  rc = pl.finish(c);
  if (rc) return rc;
  return filter ? deliver_int(c, c->scal + 1, badnum) : STDIC_OK;
}

int stdic_icgn_adjoint(stdic_ctx* c, const stdic_frame* fr, const double* coords, int N, int winsize,
                       const int32_t* ws_list, const double* U, const double* F, double* cost,
                       double* cost_n, double* dU, double* dF, void* dg, int mode, int precision) {
  if (!c) return STDIC_E_ARG;
  if (!fr || !fr->f || !fr->g || fr->W < 4 || fr->H < 4 || (fr->dtype != STDIC_F64 && fr->dtype != STDIC_F32))
    return fail(c, STDIC_E_ARG, "adjoint: bad frame (f, g and W, H >= 4 are needed)");
  if (N < 0 || (N > 0 && (!coords || !U || !F)) || (mode != STDIC_ADJ_RECOMPUTE && mode != STDIC_ADJ_STORE))
    return fail(c, STDIC_E_ARG, "adjoint: bad arguments");
  if (precision != STDIC_PLAIN_F64 && precision != STDIC_BATCHED_F32)
    return fail(c, STDIC_E_ARG, "unknown precision");
  if (precision == STDIC_PLAIN_F64 && fr->dtype != STDIC_F64)
    return fail(c, STDIC_E_ARG, "adjoint: FP64 precision needs double images");
  if (!ws_list && (winsize < 0 || (winsize & 1)))
    return fail(c, STDIC_E_ARG, "adjoint: winsize must be even and >= 0");
  cudaSetDevice(c->device);
  const bool f64 = precision == STDIC_PLAIN_F64;
  // largest subset size (read on the host; the list is small)
  int ws_max = winsize;
  if (ws_list && N > 0) {
    std::vector<int32_t> wl((size_t)N);
    if (is_device_ptr(ws_list)) {
      cudaError_t e = cudaMemcpyAsync(wl.data(), ws_list, sizeof(int32_t) * N, cudaMemcpyDeviceToHost, c->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
      if (e != cudaSuccess) return cuda_fail(c, e, "adjoint: subset sizes");
    } else {
      std::memcpy(wl.data(), ws_list, sizeof(int32_t) * N);
    }
    ws_max = 0;
    for (int32_t w : wl) {
      if (w < 0 || (w & 1) || w > 1024) return fail(c, STDIC_E_ARG, "adjoint: subset sizes must be even, 0..1024");
      ws_max = std::max(ws_max, (int)w);
    }
  }
  if (ws_max > 1024) return fail(c, STDIC_E_ARG, "adjoint: subset size above 1024");
  const size_t np = (size_t)fr->W * fr->H;
  const size_t es_in = fr->dtype == STDIC_F64 ? 8 : 4, es = f64 ? 8 : 4;
  Plan pl;
  stdic::AdjointArgs a{};
  const unsigned char *fin = nullptr, *gin = nullptr;
  pl.in((const unsigned char*)fr->f, es_in * np, (unsigned char**)&fin);
  pl.in((const unsigned char*)fr->g, es_in * np, (unsigned char**)&gin);
  pl.in(fr->mask, fr->mask ? np : 0, (uint8_t**)&a.mask);
  pl.in(coords, 2 * (size_t)N, (double**)&a.coords);
  pl.in(U, 2 * (size_t)N, (double**)&a.U);
  pl.in(F, 4 * (size_t)N, (double**)&a.F);
  pl.in(ws_list, (size_t)N, (int32_t**)&a.ws_list);
  pl.out_opt(cost_n, (size_t)std::max(N, 1), &a.cost_n);
  pl.out(cost, 1, &a.cost);
  pl.out(dU, 2 * (size_t)N, &a.dU);
  pl.out(dF, 4 * (size_t)N, &a.dF);
  unsigned char* dgp = nullptr;
  pl.out((unsigned char*)dg, dg ? es * np : 0, &dgp);
  float *f32 = nullptr, *g32 = nullptr;
  const bool convert = !f64 && fr->dtype == STDIC_F64;
  if (convert) {
    pl.scratch(np, &f32);
    pl.scratch(np, &g32);
  }
  int rc = pl.commit(c);
  if (rc) return rc;
  if (convert) {
    rc = check_launch(c, stdic::launch_to_f32((const double*)fin, f32, (long long)np, c->stream), "to_f32");
    if (!rc) rc = check_launch(c, stdic::launch_to_f32((const double*)gin, g32, (long long)np, c->stream), "to_f32");
    if (rc) return rc;
    a.f = f32; a.g = g32;
  } else {
    a.f = fin; a.g = gin;
  }
  a.W = fr->W; a.H = fr->H; a.N = N;
  a.ws_all = winsize; a.ws_max = ws_max;
  a.dg = dgp;
  a.head = c->scal + 7;
  a.f64 = f64 ? 1 : 0;
  a.store = mode == STDIC_ADJ_STORE ? 1 : 0;
  a.nsm = c->nsm;
  long long nl = 0;
  cudaEventRecord(c->es0, c->stream);
  cudaError_t e = stdic::launch_adjoint(a, c->stream, &nl);
  cudaEventRecord(c->es1, c->stream);
  c->launches += nl;
  if (e != cudaSuccess) return cuda_fail(c, e, "adjoint");
  c->solver_timed = true;
  return pl.finish(c);
}

int stdic_nodal_strain(stdic_ctx* c, const double* coords, int N, const int32_t* elems, int E,
                       const double* U, int gauss_order, double* F) {
  if (!c) return STDIC_E_ARG;
  if (N < 0 || E < 0 || (N > 0 && (!coords || !U || !F)) || (E > 0 && !elems) || gauss_order < 2 ||
      gauss_order > 5)
    return fail(c, STDIC_E_ARG, "nodal strain: bad arguments (GaussPtOrder 2..5)");
  cudaSetDevice(c->device);
  Plan pl;
  const double *dc = nullptr, *du = nullptr;
  const int32_t* de = nullptr;
  double* dF = nullptr;
  unsigned char* tws = nullptr;
  pl.in(coords, 2 * (size_t)N, (double**)&dc);
  pl.in(elems, 8 * (size_t)E, (int32_t**)&de);
  pl.in(U, 2 * (size_t)N, (double**)&du);
  pl.out(F, 4 * (size_t)N, &dF);
  pl.scratch(stdic::topo_workspace_bytes(N, E), &tws);
  int rc = pl.commit(c);
  if (rc) return rc;
  if (N > 0) {
    int *ptr = nullptr, *list = nullptr;
    rc = check_launch(c, stdic::build_topology(de, E, N, tws, &ptr, &list, c->stream), "mesh topology", E > 0 ? 4 : 2);
    if (!rc) rc = check_launch(c, stdic::launch_nodal_strain(dc, N, de, E, du, gauss_order, ptr, list, dF, c->stream),
                               "nodal strain");
    if (rc) return rc;
  }
  return pl.finish(c);
}

int stdic_fill_nans(stdic_ctx* c, const double* coords, int N, const int32_t* elems, int E, double* U) {
  if (!c) return STDIC_E_ARG;
  if (N < 0 || E < 0 || (N > 0 && !U) || (E > 0 && !elems))
    return fail(c, STDIC_E_ARG, "NaN fill: bad arguments");
  (void)coords;
  cudaSetDevice(c->device);
  Plan pl;
  const double* uin = nullptr;
  double* uout = nullptr;
  const int32_t* de = nullptr;
  double* tmp = nullptr;
  unsigned char* tws = nullptr;
  pl.in(elems, 8 * (size_t)E, (int32_t**)&de);
  pl.in((const double*)U, 2 * (size_t)N, (double**)&uin);
  pl.out(U, 2 * (size_t)N, &uout);
  pl.scratch(stdic::fill_tmp_doubles(std::max(N, 1)), &tmp);
  pl.scratch(stdic::topo_workspace_bytes(N, E), &tws);
  int rc = pl.commit(c);
  if (rc) return rc;
  if (N > 0) {
    if (uin != uout) {
      cudaError_t e = cudaMemcpyAsync(uout, uin, 16 * (size_t)N, cudaMemcpyDeviceToDevice, c->stream);
      if (e != cudaSuccess) return cuda_fail(c, e, "NaN fill");
    }
    int *ptr = nullptr, *list = nullptr;
    rc = check_launch(c, stdic::build_topology(de, E, N, tws, &ptr, &list, c->stream), "mesh topology", E > 0 ? 4 : 2);
    if (!rc) rc = check_launch(c, stdic::launch_fill_nans(N, de, E, ptr, list, uout, tmp, c->stream), "NaN fill", 2);
    if (rc) return rc;
  }
  return pl.finish(c);
}

int stdic_admm(stdic_ctx* c, const stdic_frame* fr, const double* coords, int N, const int32_t* elems, int E,
               const int32_t* dirichlet, int nd, const int32_t* winsize_list, const uint8_t* mark_hole,
               double mu, double beta, double tol, int steps, int precision, int use_graph, double* U2,
               double* F2, double* udual, double* vdual, double* U1, int* badnum, int* pcg_iters,
               int* graph_used) {
  if (!c) return STDIC_E_ARG;
  if (N <= 0 || E <= 0 || !frame_ok(fr) || !coords || !elems || !winsize_list || !U2 || !F2 || !udual ||
      !vdual || steps < 1 || (nd > 0 && !dirichlet) || nd < 0 || !(tol > 0))
    return fail(c, STDIC_E_ARG, "ADMM: bad arguments");
  if (precision == STDIC_PLAIN_F64 && fr->dtype != STDIC_F64)
    return fail(c, STDIC_E_ARG, "plain FP64 IC-GN needs double images");
  if (precision != STDIC_PLAIN_F64 && precision != STDIC_BATCHED_F32)
    return fail(c, STDIC_E_ARG, "unknown precision");
  cudaSetDevice(c->device);
  const bool batched = precision == STDIC_BATCHED_F32;
  int wmax = 2;
  {
    std::vector<int32_t> wl(2 * (size_t)N);
    if (is_device_ptr(winsize_list)) {
      cudaMemcpyAsync(wl.data(), winsize_list, wl.size() * 4, cudaMemcpyDeviceToHost, c->stream);
      cudaStreamSynchronize(c->stream);
    } else {
      std::memcpy(wl.data(), winsize_list, wl.size() * 4);
    }
    for (int32_t w : wl) wmax = std::max(wmax, (int)w);
  }
  if (wmax > 96) return fail(c, STDIC_E_ARG, "ADMM: winsize_List entries must be <= 96");
  const size_t n2 = 2 * (size_t)N, n4 = 4 * (size_t)N;
  Plan pl;
  FrameDev d;
  stage_frame(c, pl, fr, &d, batched, 1);
  const double* dcoords = nullptr;
  const int32_t *delems = nullptr, *ddir = nullptr, *dwl = nullptr;
  const uint8_t* dmark = nullptr;
  pl.in(coords, n2, (double**)&dcoords);
  pl.in(elems, 8 * (size_t)E, (int32_t**)&delems);
  pl.in(dirichlet, (size_t)nd, (int32_t**)&ddir);
  pl.in(winsize_list, n2, (int32_t**)&dwl);
  pl.in(mark_hole, mark_hole ? (size_t)N : 0, (uint8_t**)&dmark);
  // in/out state: read at the start, written at the end
  const double *iU2 = nullptr, *iF2 = nullptr, *iud = nullptr, *ivd = nullptr;
  double *oU2 = nullptr, *oF2 = nullptr, *oud = nullptr, *ovd = nullptr, *oU1 = nullptr;
  pl.in((const double*)U2, n2, (double**)&iU2);
  pl.in((const double*)F2, n4, (double**)&iF2);
  pl.in((const double*)udual, n4, (double**)&iud);
  pl.in((const double*)vdual, n2, (double**)&ivd);
  pl.out(U2, n2, &oU2);
  pl.out(F2, n4, &oF2);
  pl.out(udual, n4, &oud);
  pl.out(vdual, n2, &ovd);
  pl.out_opt(U1, n2, &oU1);
  int *hbad = nullptr, *hit = nullptr, *hst = nullptr, *dsc = nullptr;
  pl.out_opt(badnum, (size_t)steps, &hbad);
  pl.out_opt(pcg_iters, (size_t)steps, &hit);
  pl.scratch((size_t)steps, &hst);
  pl.scratch(16, &dsc);  // [0] badnum, [1] iters, [2] status, [4..13] bad-point code statistics (5 x int64)
  double *F1 = nullptr, *tmp = nullptr, *dres = nullptr;
  int32_t* conv = nullptr;
  pl.scratch(n4, &F1);
  pl.scratch(stdic::fill_tmp_doubles(N), &tmp);
  pl.scratch(8, &dres);
  pl.scratch((size_t)N, &conv);
  unsigned char *tws = nullptr, *sws = nullptr, *bscr = nullptr;
  pl.scratch(stdic::topo_workspace_bytes(N, E), &tws);
  pl.scratch(stdic::subpb2_workspace_bytes(N, E), &sws);
  int32_t* order = nullptr;
  const int npx_max = stdic::grown_tile_pixels(wmax);
  std::vector<BatchedCand> cands;
  pl.scratch((size_t)N, &order);
  if (batched) {
    cands = batched_candidates(c, true, npx_max, N);
    pl.scratch(batched_scratch_need(cands), &bscr);
  }
  int rc = pl.commit(c);
  if (rc) return rc;
  auto copy_in = [&](double* dst, const double* src, size_t n) -> int {
    if (dst == src) return STDIC_OK;
    const cudaError_t e = cudaMemcpyAsync(dst, src, 8 * n, cudaMemcpyDeviceToDevice, c->stream);
    return e == cudaSuccess ? STDIC_OK : cuda_fail(c, e, "ADMM state");
  };
  rc = copy_in(oU2, iU2, n2);
  if (!rc) rc = copy_in(oF2, iF2, n4);
  if (!rc) rc = copy_in(oud, iud, n4);
  if (!rc) rc = copy_in(ovd, ivd, n2);
  if (!rc && batched) rc = convert_frame(c, fr, &d, 1);
  int *ptr = nullptr, *list = nullptr;
  if (!rc) rc = check_launch(c, stdic::build_topology(delems, E, N, tws, &ptr, &list, c->stream), "mesh topology", E > 0 ? 4 : 2);
  if (rc) return rc;

  // Subpb1 (2-DOF IC-GN): UOld = U2, FOld = F2 -> U1
  stdic::IcgnArgs a{};
  a.f = d.f; a.g = d.g; a.mask = d.mask; a.dfdx = d.dfdx; a.dfdy = d.dfdy;
  a.W = fr->W; a.H = fr->H; a.N = N; a.mu = mu; a.tol = tol; a.ws_max = wmax; a.npx_max = npx_max;
  a.coords = dcoords; a.UOld = oU2; a.FOld = oF2; a.vdual = ovd; a.wsl2 = dwl; a.U = oU1; a.conv = conv;
  stdic::BatchedArgs b{};
  b.a = a;
  b.f32 = d.f32; b.g32 = d.g32; b.dfdx32 = d.dfdx32; b.dfdy32 = d.dfdy32;
  b.order = order; b.two_dof = 1; b.frames = 1; b.g_stride = 0; b.scratch = bscr;
  // Subpb2: (U1, F1) -> U2
  stdic::Subpb2Args s2{};
  s2.coords = dcoords; s2.N = N; s2.elems = delems; s2.E = E; s2.dirichlet = ddir; s2.nd = nd;
  s2.neumann = nullptr; s2.nn = 0; s2.gauss_order = 2; s2.beta = beta; s2.mu = mu; s2.alpha = 0.0;
  s2.winstepsize = 1.0; s2.U = oU1; s2.F = F1; s2.tol = 1e-10; s2.maxit = 10000; s2.Uhat = oU2;
  s2.spin_limit = c->wait_limit;

  auto body = [&]() -> int {
    int r = STDIC_OK;
    if (batched) r = run_batched(c, b, N, cands, QueueKeys{nullptr, dwl, 0});
    else {
      int nk = 0;
      r = check_launch(c, stdic::launch_icgn2_plain(a, order, c->scal + 64, c->scal + 12, c->stream, &nk, &c->plain),
                       "Subpb1 plain", 0);
      c->launches += nk;
    }
    if (!r) r = check_launch(c, stdic::launch_badpoints(conv, N, oU1, nullptr, 1, dsc, (unsigned long long*)(dsc + 4), c->stream), "bad points", 2);
    if (!r) r = check_launch(c, stdic::launch_fill_nans(N, delems, E, ptr, list, oU1, tmp, c->stream), "NaN fill", 2);
    if (!r) {
      const cudaError_t e = cudaMemcpyAsync(F1, oF2, 8 * n4, cudaMemcpyDeviceToDevice, c->stream);
      if (e != cudaSuccess) r = cuda_fail(c, e, "FSubpb1");
    }
    if (!r) r = check_launch(c, stdic::launch_copy_marked(dmark, N, 2, oU2, oU1, c->stream), "hole copy");
    if (!r) {
      long long nl = 0;
      const cudaError_t e =
          stdic::run_subpb2(s2, sws, dsc + 1, dres, dsc + 2, c->stream, &nl, stdic::kSubpb2Solve);
      c->launches += nl;
      if (e != cudaSuccess) r = cuda_fail(c, e, "Subpb2");
    }
    if (!r) r = check_launch(c, stdic::launch_nodal_strain(dcoords, N, delems, E, oU2, 2, ptr, list, oF2, c->stream),
                             "nodal strain");
    if (!r) r = check_launch(c, stdic::launch_copy_marked(dmark, N, 4, F1, oF2, c->stream), "hole copy");
    if (!r) r = check_launch(c, stdic::launch_copy_marked(dmark, N, 2, oU1, oU2, c->stream), "hole copy");
    if (!r) r = check_launch(c, stdic::launch_sub(oF2, F1, oud, (long long)n4, c->stream), "dual update");
    if (!r) r = check_launch(c, stdic::launch_sub(oU2, oU1, ovd, (long long)n2, c->stream), "dual update");
    return r;
  };
  auto record = [&](int step) -> int {
    cudaError_t e = cudaMemcpyAsync(hbad + step, dsc, sizeof(int), cudaMemcpyDeviceToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hit + step, dsc + 1, sizeof(int), cudaMemcpyDeviceToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hst + step, dsc + 2, sizeof(int), cudaMemcpyDeviceToDevice, c->stream);
    return e == cudaSuccess ? STDIC_OK : cuda_fail(c, e, "ADMM history");
  };

  // the Subpb2 structure (mesh graph, CSR pattern, Dirichlet flags) is the
  // same in every iteration: built once here
  {
    long long nl = 0;
    const cudaError_t e =
        stdic::run_subpb2(s2, sws, dsc + 1, dres, dsc + 2, c->stream, &nl, stdic::kSubpb2Structure);
    c->launches += nl;
    if (e != cudaSuccess) return cuda_fail(c, e, "Subpb2 structure");
  }
  // the first iteration runs directly (it tunes the batched launch shape);
  // the others replay one captured graph of the iteration
  rc = body();
  if (!rc) rc = record(0);
  if (rc) return rc;
  bool graphed = false;
  cudaGraphExec_t exec = nullptr;
  if (use_graph && steps > 1) {
    cudaGraph_t graph = nullptr;
    const long long l0 = c->launches;
    cudaError_t e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      c->capturing = true;
      const int r = body();
      c->capturing = false;
      e = cudaStreamEndCapture(c->stream, &graph);
      if (r == STDIC_OK && e == cudaSuccess && graph)
        e = cudaGraphInstantiate(&exec, graph, 0);
      if (graph) cudaGraphDestroy(graph);
      graphed = r == STDIC_OK && e == cudaSuccess && exec;
    }
    const long long per = c->launches - l0;
    c->launches = l0;
    if (!graphed) {
      cudaGetLastError();
      if (exec) { cudaGraphExecDestroy(exec); exec = nullptr; }
    } else {
      for (int step = 1; step < steps && !rc; ++step) {
        e = cudaGraphLaunch(exec, c->stream);
        if (e != cudaSuccess) rc = cuda_fail(c, e, "ADMM graph launch");
        else { c->launches += per; rc = record(step); }
      }
      cudaGraphExecDestroy(exec);
    }
  }
  if (!graphed)
    for (int step = 1; step < steps && !rc; ++step) {
      rc = body();
      if (!rc) rc = record(step);
    }
  if (graph_used) *graph_used = graphed ? 1 : 0;
  if (rc) return rc;
  rc = pl.finish(c);
  if (rc) return rc;
  std::vector<int> st((size_t)steps);
  cudaError_t e = cudaMemcpyAsync(st.data(), hst, sizeof(int) * steps, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "ADMM status");
  for (int v : st) {
    if (v == 2) return fail(c, STDIC_E_TIMEOUT, "ADMM: Subpb2 grid barrier wait gave up");
    if (v == 3) return fail(c, STDIC_E_ARG, "ADMM: invalid node index or node in >16 elements");
    if (v == 1) return fail(c, STDIC_E_NOTCONV, "ADMM: Subpb2 PCG did not reach the tolerance");
  }
  return STDIC_OK;
}

int stdic_subpb2(stdic_ctx* c, const double* coords, int N, const int32_t* elems, int E,
                 const int32_t* dirichlet, int nd, const double* neumann, int nn, int gauss_order,
                 double beta, double mu, const double* U, const double* F, double alpha, double winstepsize,
                 double tol, int maxit, double* Uhat, int* iters) {
  if (!c) return STDIC_E_ARG;
  if (N < 0 || E < 0 || nd < 0 || nn < 0 || (N > 0 && (!coords || !U || !F || !Uhat)) ||
      (E > 0 && !elems) || (nd > 0 && !dirichlet) || (nn > 0 && !neumann) || gauss_order < 2 ||
      gauss_order > 5 || (nn > 0 && !(winstepsize != 0)))
    return fail(c, STDIC_E_ARG, "Subpb2Quadtree: bad arguments (GaussPtOrder 2..5)");
  cudaSetDevice(c->device);
  Plan pl;
  stdic::Subpb2Args a{};
  pl.in(coords, 2 * (size_t)N, (double**)&a.coords);
  pl.in(elems, 8 * (size_t)E, (int32_t**)&a.elems);
  pl.in(dirichlet, (size_t)nd, (int32_t**)&a.dirichlet);
  pl.in(neumann, 4 * (size_t)nn, (double**)&a.neumann);
  pl.in(U, 2 * (size_t)N, (double**)&a.U);
  pl.in(F, 4 * (size_t)N, (double**)&a.F);
  pl.out(Uhat, 2 * (size_t)N, &a.Uhat);
  unsigned char* wsp = nullptr;
  pl.scratch(stdic::subpb2_workspace_bytes(N, E), &wsp);
  int rc = pl.commit(c);
  if (rc) return rc;
  a.N = N; a.E = E; a.nd = nd; a.nn = nn; a.gauss_order = gauss_order;
  a.beta = beta; a.mu = mu; a.alpha = alpha; a.winstepsize = winstepsize;
  a.tol = tol > 0 ? tol : 1e-10;
  a.maxit = maxit > 0 ? maxit : 10000;
  a.spin_limit = c->wait_limit;
  if (N > 0) {
    long long nl = 0;
    cudaError_t e = stdic::run_subpb2(a, wsp, c->scal + 2, c->scald, c->scal + 3, c->stream, &nl);
    c->launches += nl;
    if (e != cudaSuccess) return cuda_fail(c, e, "Subpb2Quadtree");
  }
  rc = pl.finish(c);
  if (rc) return rc;
  if (N <= 0) { if (iters) *iters = 0; return STDIC_OK; }
  int hs[2] = {0, 0};
  cudaError_t e = cudaMemcpyAsync(hs, c->scal + 2, 2 * sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "Subpb2Quadtree status");
  if (iters) {
    if (is_device_ptr(iters)) cudaMemcpyAsync(iters, c->scal + 2, sizeof(int), cudaMemcpyDeviceToDevice, c->stream);
    else *iters = hs[0];
  }
  if (hs[1] == 2) return fail(c, STDIC_E_TIMEOUT, "Subpb2Quadtree: grid barrier wait gave up");
  if (hs[1] == 3) return fail(c, STDIC_E_ARG, "Subpb2Quadtree: invalid node index or node in >16 elements");
  if (hs[1] == 1) return fail(c, STDIC_E_NOTCONV, "Subpb2Quadtree: PCG did not reach the tolerance");
  return STDIC_OK;
}


// ---------------------------------------------------------------------------
// GenerateQuadtreeMesh.m:18-133 on the uniform mesh of MeshSetUp.m.
int stdic_quadtree_mesh(stdic_ctx* c, const uint8_t* mask, int W, int H, const double* x0, const double* y0,
                        int ny, int nx, double winstepsize, double element_min_size, double* coords,
                        int32_t* elems, int32_t* irregular, int32_t* dirichlet, const int64_t* capacity,
                        int64_t* counts) {
  if (!c) return STDIC_E_ARG;
  if (!mask || W < 1 || H < 1 || !x0 || !y0 || ny < 2 || nx < 2 || !(winstepsize > 0) || !counts ||
      ((coords || elems || irregular || dirichlet) && !capacity))
    return fail(c, STDIC_E_ARG, "GenerateQuadtreeMesh: bad arguments (a grid of at least 2 x 2, step > 0)");
  cudaSetDevice(c->device);
  Plan pl;
  const uint8_t* dm;
  pl.in(mask, (size_t)W * H, (uint8_t**)&dm);
  int rc = pl.commit(c);
  if (rc) return rc;
  // the grids are read on the host
  const size_t ng = (size_t)nx * ny;
  std::vector<double> gx(ng), gy(ng);
  for (int k = 0; k < 2; ++k) {
    const double* src = k ? y0 : x0;
    double* dst = k ? gy.data() : gx.data();
    if (is_device_ptr(src)) {
      cudaError_t e = cudaMemcpyAsync(dst, src, ng * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
      if (e != cudaSuccess) return cuda_fail(c, e, "GenerateQuadtreeMesh grid read");
    } else {
      std::memcpy(dst, src, ng * sizeof(double));
    }
  }
  for (size_t k = 0; k < ng; ++k)
    if (!std::isfinite(gx[k]) || !std::isfinite(gy[k]) || gx[k] != std::floor(gx[k]) || gy[k] != std::floor(gy[k]))
      return fail(c, STDIC_E_ARG, "GenerateQuadtreeMesh: grid positions must be whole pixels");
  auto grow = [c](size_t bytes) -> void* {
    if (bytes > c->aux_size) {
      if (c->aux) {
        cudaStreamSynchronize(c->stream);
        cudaFree(c->aux);
        c->aux = nullptr;
        c->aux_size = 0;
      }
      const size_t want = std::max(bytes, c->aux_size * 2);
      if (cudaMalloc(&c->aux, want) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
      }
      c->aux_size = want;
    }
    return c->aux;
  };
  stdic::QuadtreeMeshOut out;
  const char* err = nullptr;
  rc = stdic::quadtree_mesh_generate(dm, W, H, gx.data(), gy.data(), ny, nx, winstepsize, element_min_size, &out,
                                     grow, c->stream, &c->launches, &err);
  if (rc) return fail(c, rc, std::string("GenerateQuadtreeMesh: ") + (err ? err : "failed"));
  const int64_t N = (int64_t)out.x.size(), E = (int64_t)out.elems.size(), nI = (int64_t)out.irregular.size(),
                nd = (int64_t)out.dirichlet.size();
  counts[0] = N; counts[1] = E; counts[2] = nI; counts[3] = nd;
  const int64_t need[4] = {N, E, nI, nd};
  void* const dst[4] = {coords, elems, irregular, dirichlet};
  for (int k = 0; k < 4; ++k)
    if (dst[k] && capacity[k] < need[k])
      return fail(c, STDIC_E_ARG, "GenerateQuadtreeMesh: an output holds fewer rows than the mesh (see counts)");
  // column-major host images of the outputs, then one copy each
  std::vector<double> hc((size_t)2 * N);
  for (int64_t k = 0; k < N; ++k) { hc[k] = out.x[k]; hc[N + k] = out.y[k]; }
  std::vector<int32_t> he((size_t)8 * E), hi((size_t)3 * nI), hd(out.dirichlet.begin(), out.dirichlet.end());
  for (int64_t e = 0; e < E; ++e)
    for (int k = 0; k < 8; ++k) he[k * E + e] = out.elems[e][k];
  for (int64_t i = 0; i < nI; ++i)
    for (int k = 0; k < 3; ++k) hi[k * nI + i] = out.irregular[i][k];
  const void* src[4] = {hc.data(), he.data(), hi.data(), hd.data()};
  const size_t bytes[4] = {hc.size() * sizeof(double), he.size() * sizeof(int32_t), hi.size() * sizeof(int32_t),
                           hd.size() * sizeof(int32_t)};
  for (int k = 0; k < 4; ++k) {
    if (!dst[k] || bytes[k] == 0) continue;
    if (is_device_ptr(dst[k])) {
      cudaError_t e = cudaMemcpyAsync(dst[k], src[k], bytes[k], cudaMemcpyHostToDevice, c->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
      if (e != cudaSuccess) return cuda_fail(c, e, "GenerateQuadtreeMesh output copy");
    } else {
      std::memcpy(dst[k], src[k], bytes[k]);
    }
  }
  return STDIC_OK;
}


// ---------------------------------------------------------------------------
// funIntegerSearchMg.m: multigrid integer search, node grid chosen inside.
int stdic_integer_search_mg(stdic_ctx* c, const double* f, const double* g, int W, int H, const double gridx[2],
                            const double gridy[2], int winsize, const double winstepsize[2], double* x, double* y,
                            double* u, double* v, double* cc, int64_t capacity, int32_t counts[2],
                            double* blocks, int64_t block_capacity, int64_t* nblocks) {
  if (!c) return STDIC_E_ARG;
  if (!f || !g || W < 8 || H < 8 || !gridx || !gridy || winsize < 2 || !winstepsize || !(winstepsize[0] > 0) ||
      !(winstepsize[1] > 0) || !counts || ((x || y || u || v || cc) && capacity < 4))
    return fail(c, STDIC_E_ARG, "funIntegerSearchMg: bad arguments");
  cudaSetDevice(c->device);
  Plan pl;
  const double *df, *dg;
  unsigned char* fixed;
  pl.in(f, (size_t)W * H, (double**)&df);
  pl.in(g, (size_t)W * H, (double**)&dg);
  pl.scratch(stdic::mg_fixed_workspace_bytes(W, H), &fixed);
  int rc = pl.commit(c);
  if (rc) return rc;
  auto grow = [c](size_t bytes) -> void* {
    if (bytes > c->aux_size) {
      if (c->aux) {
        cudaStreamSynchronize(c->stream);
        cudaFree(c->aux);
        c->aux = nullptr;
        c->aux_size = 0;
      }
      const size_t want = std::max(bytes, c->aux_size * 2);
      if (cudaMalloc(&c->aux, want) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
      }
      c->aux_size = want;
    }
    return c->aux;
  };
  stdic::MgSearchOut out;
  const char* err = nullptr;
  rc = stdic::integer_search_mg(df, dg, W, H, gridx, gridy, winsize, winstepsize, fixed, grow, c->stream,
                                &c->launches, &out, &err);
  if (rc) {
    const int code = rc == -1 ? STDIC_E_ARG
                     : rc == -3 ? STDIC_E_NOMEM
                     : rc == -5 ? STDIC_E_TIMEOUT
                     : rc == -6 ? STDIC_E_NOTCONV
                                : STDIC_E_CUDA;
    return fail(c, code, std::string("funIntegerSearchMg: ") + (err ? err : "failed"));
  }
  counts[0] = out.nx;
  counts[1] = out.ny;
  if (nblocks) *nblocks = out.nblocks;
  if (blocks) {
    if (block_capacity < out.nblocks)
      return fail(c, STDIC_E_ARG, "funIntegerSearchMg: blocks holds fewer rows than the last level (see nblocks)");
    const size_t bytes = sizeof(double) * out.blocks.size();
    if (is_device_ptr(blocks)) {
      cudaError_t e = cudaMemcpyAsync(blocks, out.blocks.data(), bytes, cudaMemcpyHostToDevice, c->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
      if (e != cudaSuccess) return cuda_fail(c, e, "funIntegerSearchMg block copy");
    } else {
      std::memcpy(blocks, out.blocks.data(), bytes);
    }
  }
  const int64_t ng = (int64_t)out.nx * out.ny;
  if ((x || y || u || v || cc) && capacity < ng)
    return fail(c, STDIC_E_ARG, "funIntegerSearchMg: the outputs hold fewer elements than the node grid (see counts)");
  // ny x nx column-major (row = y), as meshgrid(xList, yList) and gridfit give them
  std::vector<double> hx(ng), hy(ng);
  for (int i = 0; i < out.nx; ++i)
    for (int j = 0; j < out.ny; ++j) {
      hx[j + (int64_t)out.ny * i] = out.xnodes[i];
      hy[j + (int64_t)out.ny * i] = out.ynodes[j];
    }
  const double* src[5] = {hx.data(), hy.data(), out.x3.data(), out.x3.data() + ng, out.x3.data() + 2 * ng};
  double* dst[5] = {x, y, u, v, cc};
  for (int k = 0; k < 5; ++k) {
    if (!dst[k]) continue;
    if (is_device_ptr(dst[k])) {
      cudaError_t e = cudaMemcpyAsync(dst[k], src[k], sizeof(double) * ng, cudaMemcpyHostToDevice, c->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
      if (e != cudaSuccess) return cuda_fail(c, e, "funIntegerSearchMg output copy");
    } else {
      std::memcpy(dst[k], src[k], sizeof(double) * ng);
    }
  }
  return STDIC_OK;
}

// ---------------------------------------------------------------------------
// funPOR_GPR.m: the next frame's field predicted from earlier frames.
int stdic_por_gpr(stdic_ctx* c, const double* T_snap, int nT, int64_t np, const double* t_train,
                  const double* t_pre, int nT1, int nB, double* u_pred, double* alpha, double* beta_pod,
                  double* beta_gpr) {
  if (!c) return STDIC_E_ARG;
  if (!T_snap || !t_train || !t_pre || !u_pred || nT < 2 || np < 2 || nT1 < 1 || nB < 1)
    return fail(c, STDIC_E_ARG, "funPOR_GPR: bad arguments");
  cudaSetDevice(c->device);
  Plan pl;
  const double* dT;
  double* dU;
  unsigned char* ws;
  pl.in(T_snap, (size_t)nT * np, (double**)&dT);
  pl.out(u_pred, (size_t)nT1 * np, &dU);
  pl.scratch(stdic::por_workspace_bytes(np, nT, nB), &ws);
  int rc = pl.commit(c);
  if (rc) return rc;
  const char* err = nullptr;
  rc = stdic::por_gpr(dT, nT, np, t_train, t_pre, nT1, nB, dU, alpha, beta_pod, beta_gpr, ws, c->stream,
                      &c->launches, &err);
  if (rc) return fail(c, rc, err ? err : "funPOR_GPR failed");
  return pl.finish(c);
}

}  // extern "C"
