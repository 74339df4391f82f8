// pg_gradient_noalloc: the cell gradient of pg_gradient without any device
// allocation, for callers that cannot call cudaMalloc.
//
// pg_gradient needs 2*n_faces doubles of scratch for the face gradients when
// the caller does not want them back, and it allocates that scratch per call.
// Some callers cannot allocate at that point: a time loop that runs inside a
// fixed device-memory budget handed out by an outer framework, or code that
// must not trigger cudaMalloc/cudaFree because those calls synchronise the
// device and stall the other work in flight.  This entry point keeps the
// scratch in one file-scope __device__ array instead.
//
// Limits and sharing:
//  * meshes of at most kNoAllocMaxFaces faces (larger ones are rejected with
//    PG_BAD_ARG); the array takes 16 MiB on every GPU that loads the library,
//    for as long as the process lives;
//  * one device: the library issues its work on one stream, created on the
//    device that was current at the library's first call, and the mesh's
//    buffers live there too; a call made with another device current, or
//    given pointers that are not device memory of that device, is rejected
//    with PG_BAD_ARG before anything is launched;
//  * the array's device address is looked up on the first call and kept;
//    make that first call before any stream capture begins;
//  * every call shares the one array and overwrites its first 2*n_faces
//    entries before reading them (nothing has to start at zero); two calls
//    whose kernels run at the same time -- e.g. issued on other streams, or
//    from several host threads -- race on it.
#include <cuda_runtime.h>

#include <mutex>

#include "internal.h"
#include "kernels.cuh"

namespace {

constexpr int64_t kNoAllocMaxFaces = (int64_t)1 << 20;

__device__ __align__(256) double g_face_grad_scratch[2 * kNoAllocMaxFaces];

std::mutex g_mu;
double *g_scratch_ptr = nullptr;  // device address of the array
int g_scratch_dev = -1;           // the device it was looked up on

// The device a pointer's memory belongs to, or -1 when it is not device or
// managed memory (a host pointer passed by mistake).
int device_of(const void *p) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();  // a failed query leaves a (non-sticky) error: clear it
    return -1;
  }
  if (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged)
    return -1;
  return at.device;
}

// Device address of the scratch array on device dev (looked up once, with
// dev current).
int scratch_on(int dev, double **out) {
  std::lock_guard<std::mutex> g(g_mu);
  if (!g_scratch_ptr) {
    void *p = nullptr;
    PG_CUDA(cudaGetSymbolAddress(&p, g_face_grad_scratch));
    g_scratch_ptr = static_cast<double *>(p);
    g_scratch_dev = dev;
  }
  PG_CHECK_ARG(g_scratch_dev == dev,
               "pg_gradient_noalloc: the library runs on one device");
  *out = g_scratch_ptr;
  return PG_OK;
}

}  // namespace

extern "C" int pg_gradient_noalloc(const pg_mesh *m, const double *phi_cell,
                                   const double *phi_face, double *grad_cell) {
  PG_CHECK_ARG(m && phi_cell && phi_face && grad_cell,
               "pg_gradient_noalloc: NULL argument");
  const pg::HostMesh &h = m->h;
  if (h.n_faces > kNoAllocMaxFaces) {
    pg::set_error("pg_gradient_noalloc: mesh has " + std::to_string(h.n_faces) +
                  " faces; the allocation-free path holds at most " +
                  std::to_string(kNoAllocMaxFaces));
    return PG_BAD_ARG;
  }
  int dev = 0;
  PG_CUDA(cudaGetDevice(&dev));
  PG_CHECK_ARG(h.n_faces == 0 || device_of(m->d.fl.p) == dev,
               "pg_gradient_noalloc: the current device is not the mesh's");
  PG_CHECK_ARG(device_of(phi_cell) == dev && device_of(phi_face) == dev &&
                   device_of(grad_cell) == dev,
               "pg_gradient_noalloc: phi_cell, phi_face and grad_cell must "
               "be device memory of the current device");
  double *scratch = nullptr;
  int rc = scratch_on(dev, &scratch);
  if (rc) return rc;
  pg::launch_gradient((int)h.n_cells, (int)h.n_faces, m->d.fl.p, m->d.fr.p,
                      m->d.fcx.p, m->d.fcy.p, m->d.cx.p, m->d.cy.p,
                      m->d.link_ptr.p, m->d.link_face.p, nullptr, nullptr,
                      m->d.fnx.p, m->d.fny.p, phi_cell, phi_face, scratch,
                      grad_cell, pg::stream());
  PG_CUDA(cudaGetLastError());
  PG_CUDA(cudaStreamSynchronize(pg::stream()));
  return PG_OK;
}
