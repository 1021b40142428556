// Subpb2Quadtree on scratch that is never allocated: a fixed device array.
//
// Who needs it.  Some callers must run the global FEM step at a point where they
// cannot ask the CUDA runtime for memory:
//   * a MEX gateway or a Python host whose caching allocator (MATLAB's gpuArray
//     pool, PyTorch's caching allocator) already holds nearly all of HBM, so a
//     fresh cudaMalloc of the CSR matrix and CG vectors fails with out-of-memory
//     although the allocator itself has room;
//   * a tight ADMM loop that cannot afford the implicit device-wide
//     synchronisation cudaFree performs, nor the latency of a first cudaMalloc;
//   * an embedded host that reserves all device memory once at start-up and
//     forbids allocation afterwards.
// stdic_subpb2 needs a context, whose creation and workspace growth allocate;
// this entry needs neither.  It runs the same assembly and Jacobi-PCG launcher
// (run_subpb2) on a file-scope __device__ array whose size is fixed at build
// time, so the only memory it uses is what the module image carries.
//
// Limits and rules of use:
//   * the array holds kStaticScratchBytes; a mesh whose assembly and CG vectors
//     need more is rejected with STDIC_E_NOMEM and a message naming both sizes;
//   * every array argument must already be device memory of the current device;
//   * one array per device: two calls in flight on one device at the same time
//     (two streams, two host threads) share it and corrupt each other's result,
//     so the caller serialises them;
//   * every call looks the array's address up with cudaGetSymbolAddress while
//     the caller's device is current (the first call on a device may load the
//     module).  Nothing is cached across calls, so a context that was torn down
//     and created again (cudaDeviceReset, a primary-context release), which can
//     reload the module at another address, is picked up by the next call;
//   * the call ends with a read-back of its status and a stream synchronise,
//     so it can never be captured into a CUDA graph: on a stream that is being
//     captured it returns STDIC_E_UNSUPPORTED without touching the stream.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>

#include "../../include/staqdic.h"
#include "kernels.h"

namespace {

constexpr size_t kStaticScratchBytes = (size_t)16 << 20;  // 16 MiB
constexpr size_t kHeaderBytes = 256;                       // device scalars, then the workspace

// [0, 256): int iters, int status, double resid; [256, end): Subpb2 workspace
__device__ __align__(256) unsigned char g_subpb2_scratch[kStaticScratchBytes];

void put_err(char* err, int err_len, const char* msg) {
  if (err && err_len > 0) {
    std::strncpy(err, msg, (size_t)err_len - 1);
    err[err_len - 1] = '\0';
  }
}

int cuda_err(char* err, int err_len, const char* where, cudaError_t e) {
  char buf[256];
  std::snprintf(buf, sizeof buf, "stdic_subpb2_noalloc: %s: %s", where, cudaGetErrorString(e));
  put_err(err, err_len, buf);
  return STDIC_E_CUDA;
}

// True when p is device (or managed) memory that the device dev can use.
bool on_device(const void* p, int dev) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (at.type == cudaMemoryTypeManaged) return true;
  return at.type == cudaMemoryTypeDevice && at.device == dev;
}

}  // namespace

extern "C" int stdic_subpb2_noalloc(const double* coords, int N, const int32_t* elems, int E,
                                    const int32_t* dirichlet, int nd, const double* neumann,
                                    int nn, int gauss_order, double beta, double mu,
                                    const double* U, const double* F, double alpha,
                                    double winstepsize, double tol, int maxit, double* Uhat,
                                    int* iters, void* cuda_stream, char* err, int err_len) {
  put_err(err, err_len, "");
  if (N < 0 || E < 0 || nd < 0 || nn < 0 || (N > 0 && (!coords || !U || !F || !Uhat)) ||
      (E > 0 && !elems) || (nd > 0 && !dirichlet) || (nn > 0 && !neumann) || gauss_order < 2 ||
      gauss_order > 5 || (nn > 0 && !(winstepsize != 0))) {
    put_err(err, err_len, "stdic_subpb2_noalloc: bad arguments (GaussPtOrder 2..5)");
    return STDIC_E_ARG;
  }
  if (iters) *iters = 0;
  if (N == 0) return STDIC_OK;

  const size_t need = stdic::subpb2_workspace_bytes(N, E);
  if (need > kStaticScratchBytes - kHeaderBytes) {
    char buf[256];
    std::snprintf(buf, sizeof buf,
                  "stdic_subpb2_noalloc: mesh of %d nodes and %d elements needs %zu bytes of "
                  "scratch; the static array holds %zu",
                  N, E, need, kStaticScratchBytes - kHeaderBytes);
    put_err(err, err_len, buf);
    return STDIC_E_NOMEM;
  }

  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_err(err, err_len, "cudaGetDevice", e);
  cudaStream_t s = (cudaStream_t)cuda_stream;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  e = cudaStreamIsCapturing(s, &cap);
  if (e != cudaSuccess) return cuda_err(err, err_len, "cudaStreamIsCapturing", e);
  if (cap != cudaStreamCaptureStatusNone) {
    put_err(err, err_len,
            "stdic_subpb2_noalloc: the stream is being captured; this entry synchronises its "
            "stream and cannot be part of a CUDA graph");
    return STDIC_E_UNSUPPORTED;
  }
  // The array's device address in the current device's context, looked up on
  // every call (a host-side table lookup once the module is loaded).  The
  // symbol itself is only a host-side stand-in and is never passed to a kernel.
  unsigned char* base = nullptr;
  {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_subpb2_scratch);
    if (e != cudaSuccess) return cuda_err(err, err_len, "cudaGetSymbolAddress", e);
    base = (unsigned char*)p;
  }

  const void* arrays[] = {coords, elems, dirichlet, neumann, U, F, Uhat};
  const int counts[] = {N, E, nd, nn, N, N, N};
  for (int k = 0; k < 7; ++k) {
    if (counts[k] > 0 && !on_device(arrays[k], dev)) {
      put_err(err, err_len,
              "stdic_subpb2_noalloc: every array must be device memory of the current device");
      return STDIC_E_ARG;
    }
  }

  int* iters_dev = (int*)base;
  int* status_dev = (int*)base + 1;
  double* resid_dev = (double*)(base + 8);
  // The workspace is initialised by the launcher's own set-up kernels; the
  // scalars it only writes at the end start at zero here.
  e = cudaMemsetAsync(base, 0, kHeaderBytes, s);
  if (e != cudaSuccess) return cuda_err(err, err_len, "clear scalars", e);

  stdic::Subpb2Args a{};
  a.coords = coords; a.N = N;
  a.elems = elems; a.E = E;
  a.dirichlet = dirichlet; a.nd = nd;
  a.neumann = neumann; a.nn = nn;
  a.gauss_order = gauss_order;
  a.beta = beta; a.mu = mu; a.alpha = alpha; a.winstepsize = winstepsize;
  a.U = U; a.F = F;
  a.tol = tol > 0 ? tol : 1e-10;
  a.maxit = maxit > 0 ? maxit : 10000;
  a.Uhat = Uhat;
  e = stdic::run_subpb2(a, base + kHeaderBytes, iters_dev, resid_dev, status_dev, s, nullptr);
  if (e != cudaSuccess) return cuda_err(err, err_len, "Subpb2 launch", e);

  int hs[2] = {0, 0};
  e = cudaMemcpyAsync(hs, base, sizeof hs, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_err(err, err_len, "status read-back", e);
  if (iters) *iters = hs[0];
  if (hs[1] == 2) {
    put_err(err, err_len, "stdic_subpb2_noalloc: grid barrier wait gave up");
    return STDIC_E_TIMEOUT;
  }
  if (hs[1] == 3) {
    put_err(err, err_len, "stdic_subpb2_noalloc: invalid node index or node in >16 elements");
    return STDIC_E_ARG;
  }
  if (hs[1] == 1) {
    put_err(err, err_len, "stdic_subpb2_noalloc: PCG did not reach the tolerance");
    return STDIC_E_NOTCONV;
  }
  return STDIC_OK;
}
