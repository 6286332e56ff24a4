// fvc_api.cu -- the C ABI of include/fvc.h: contexts, device-resident mesh
// and frames, step-level calls and the FTLE / tracer jobs.
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "fvc.h"
#include "fvc_fpmath.cuh"
#include "fvc_internal.h"

void job_events(fvc_job* j) {
  for (int k = 0; k < 4; k++)
    if (!j->ev[k]) cudaEventCreate(&j->ev[k]);
}

float ev_ms(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) ms = 0.f;
  return ms;
}

// ------------------------------------------------------------------ helpers

fvc_status fail(fvc_ctx* c, fvc_status code, const char* fmt, ...) {
  if (c) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    c->err = buf;
  }
  return code;
}


fvc_status use_device(fvc_ctx* c) {
  FVC_CUDA(c, cudaSetDevice(c->device));
  return FVC_OK;
}

fvc_status check_launch(fvc_ctx* c, const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(c, FVC_ERR_CUDA, "%s launch: %s", what, cudaGetErrorString(e));
  return FVC_OK;
}

// Reads and clears the counters; maps device fault bits to a status.
static fvc_status finish(fvc_ctx* c, const char* what, long long* steps, DevCounters* out = nullptr) {
  DevCounters h{};
  FVC_CUDA(c, cudaMemcpyAsync(&h, c->d_ctr, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  FVC_CUDA(c, cudaStreamSynchronize(c->stream));
  if (steps) *steps = (long long)(h.steps + h.steps_early);
  if (out) *out = h;
  FVC_CUDA(c, cudaMemsetAsync(c->d_ctr, 0, sizeof(DevCounters), c->stream));
  if (h.status & PT_ERR_STATE)
    return fail(c, FVC_ERR_STATE, "%s: a point that had left the domain was advected", what);
  if (h.status & PT_ERR_TLOC)
    return fail(c, FVC_ERR_TLOC, "%s: query time outside the loaded frame interval", what);
  if (h.status & PT_ERR_WALK)
    return fail(c, FVC_ERR_WALK, "%s: neighbour walk failed (indeterminate neighbour or hop cap)", what);
  if (h.status & PT_ERR_CET)
    return fail(c, FVC_ERR_WALK, "%s: exposure time: a step started outside the velocity domain", what);
  return FVC_OK;
}

static fvc_status ensure_scratch(fvc_ctx* c, size_t bytes) {
  if (bytes <= c->scratch_bytes) return FVC_OK;
  if (c->d_scratch) cudaFree(c->d_scratch);
  c->d_scratch = nullptr;
  c->scratch_bytes = 0;
  if (cudaMalloc(&c->d_scratch, bytes) != cudaSuccess)
    return fail(c, FVC_ERR_OOM, "could not allocate %zu bytes of device scratch", bytes);
  c->scratch_bytes = bytes;
  return FVC_OK;
}

static inline size_t al256(size_t b) { return (b + 255) & ~(size_t)255; }

// Frees the quantised frames (their node count changed with the mesh).
static void drop_quantised(fvc_ctx* c) {
  for (auto& kv : c->qframes) cudaFree(kv.second.q);
  c->qframes.clear();
  for (auto& kv : c->qpairs) cudaFree(kv.second.q);
  c->qpairs.clear();
  c->qpair_bytes = 0;
  cudaFree(c->d_qpair);
  c->d_qpair = nullptr;
  c->window_set = false;
}

// (X, c) float pairs copied to the host back to FP64 positions X - c.
void unpack_host(double* A, size_t n) {
  for (size_t i = 0; i < n; i++) {
    float p[2];
    memcpy(p, &A[i], sizeof(p));
    A[i] = (double)p[0] - (double)p[1];
  }
}

// ------------------------------------------------------------------ context

static void out_free(fvc_ctx* c);

extern "C" int fvc_abi_version(void) { return FVC_ABI_VERSION; }

extern "C" fvc_status fvc_create(fvc_ctx** out, const fvc_opts* o) {
  if (!out || !o) return FVC_ERR_ARG;
  *out = nullptr;
  if ((o->dims != 2 && o->dims != 3) || (o->mesh_type != 0 && o->mesh_type != 1)) return FVC_ERR_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return FVC_ERR_CUDA;
  if (o->device < 0 || o->device >= ndev) return FVC_ERR_ARG;
  fvc_ctx* c = new fvc_ctx();
  c->device = o->device;
  c->mesh.dims = o->dims;
  c->mesh.mesh_type = o->mesh_type;
  c->mesh.max_hops = o->max_hops > 0 ? o->max_hops : 65536;
  for (int a = 0; a < 3; a++) {
    c->mesh.bounds[2 * a] = -1e300;
    c->mesh.bounds[2 * a + 1] = 1e300;
  }
  if (cudaSetDevice(c->device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc(&c->d_ctr, sizeof(DevCounters)) != cudaSuccess ||
      cudaMemset(c->d_ctr, 0, sizeof(DevCounters)) != cudaSuccess) {
    fvc_destroy(c);
    return FVC_ERR_CUDA;
  }
  *out = c;
  return FVC_OK;
}

extern "C" void fvc_destroy(fvc_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (auto& kv : c->frames) cudaFree(kv.second);
  for (auto& kv : c->qframes) cudaFree(kv.second.q);
  for (auto& kv : c->qpairs) cudaFree(kv.second.q);
  cudaFree(c->d_qscratch);
  cudaFree(c->d_qpair);
  cudaFree(c->d_steps);
  cudaFreeHost(c->h_ring);
  cudaFree(c->d_ring);
  for (auto& kv : c->pool) cudaFree(kv.second);
  for (auto& ev : c->ring_ev) cudaEventDestroy(ev);
  cudaFree(c->d_elem);
  cudaFree(c->d_geom);
  cudaFree(c->d_geo32);
  cudaFree(c->d_nodes);
  cudaFree(c->d_cell_start);
  cudaFree(c->d_cell_ids);
  cudaFree(c->d_stage);
  cudaFree(c->d_ctr);
  cudaFree(c->d_scratch);
  cudaFree(c->d_vt);
  cudaFree(c->d_cet_sum);
  cudaFree(c->d_cet_enc);
  out_free(c);
  if (c->up_stream) {
    cudaStreamSynchronize(c->up_stream);
    cudaStreamDestroy(c->up_stream);
  }
  for (auto& kv : c->frame_ev) cudaEventDestroy(kv.second);
  if (c->up_after) cudaEventDestroy(c->up_after);
  cudaFree(c->d_up_stage[0]);
  cudaFree(c->d_up_stage[1]);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

extern "C" const char* fvc_last_error(const fvc_ctx* c) { return c ? c->err.c_str() : "null context"; }

// ---------------------------------------------------------------- mesh

extern "C" fvc_status fvc_set_cart_mesh(fvc_ctx* c, double xmin, double xmax, int xres, double ymin,
                                        double ymax, int yres, double zmin, double zmax, int zres) {
  if (!c) return FVC_ERR_ARG;
  if (c->mesh.mesh_type != 0) return fail(c, FVC_ERR_STATE, "context is not Cartesian");
  // derived parameters as ompVC/mesh.c:101-121
  if (xres < 2 || xmin >= xmax) return fail(c, FVC_ERR_ARG, "Insufficient resolution of velocity data in x-direction");
  if (yres < 2 || ymin >= ymax) return fail(c, FVC_ERR_ARG, "Insufficient resolution of velocity data in y-direction");
  DevMesh& m = c->mesh;
  m.xmin = xmin; m.xres = xres; m.dx = (xmax - xmin) / (xres - 1);
  m.ymin = ymin; m.yres = yres; m.dy = (ymax - ymin) / (yres - 1);
  if (m.dims == 3) {
    if (zres < 2 || zmin >= zmax) return fail(c, FVC_ERR_ARG, "Insufficient resolution of velocity data in z-direction");
    m.zmin = zmin; m.zres = zres; m.dz = (zmax - zmin) / (zres - 1);
  } else {
    m.zmin = 0; m.zres = 1; m.dz = 0;
  }
  m.rdx = rcp_for_div(m.dx);
  m.rdy = rcp_for_div(m.dy);
  m.rdz = rcp_for_div(m.dz);
  long nn = (long)m.xres * m.yres * m.zres;
  if (c->frame_nodes && c->frame_nodes != nn) {
    for (auto& kv : c->frames) cudaFree(kv.second);
    c->frames.clear();
    drop_quantised(c);
  }
  c->frame_nodes = nn;
  c->mesh_set = true;
  return FVC_OK;
}

// Cells of the global-search bucket grid at most (about two elements a cell;
// FVC_BUCKET_MAX_CELLS lowers the cap, e.g. to bound the grid's memory).
static long bucket_cell_cap() {
  const long dflt = 1L << 26;
  const char* e = getenv("FVC_BUCKET_MAX_CELLS");
  if (!e || !*e) return dflt;
  char* end = nullptr;
  long v = strtol(e, &end, 10);
  return (end && *end == 0 && v > 0 && v < dflt) ? v : dflt;
}

extern "C" fvc_status fvc_set_unstruct_mesh(fvc_ctx* c, int nnodes, const double* xyz, int nelem,
                                            const int* conn, const int* adj) {
  if (!c) return FVC_ERR_ARG;
  if (c->mesh.mesh_type != 1) return fail(c, FVC_ERR_STATE, "context is not unstructured");
  if (nnodes <= 0 || nelem <= 0 || !xyz || !conn || !adj) return fail(c, FVC_ERR_ARG, "empty mesh");
  fvc_status st;
  if ((st = use_device(c))) return st;
  const int nv = c->mesh.dims == 3 ? 4 : 3;
  std::vector<double4_32a> hn((size_t)nnodes);
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (long i = 0; i < nnodes; i++) {
    hn[i] = make_double4_32a(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], 0.0);
    for (int a = 0; a < 3; a++) {
      lo[a] = fmin(lo[a], xyz[3 * i + a]);
      hi[a] = fmax(hi[a], xyz[3 * i + a]);
    }
  }
  // Everything of the new mesh -- records, nodes and bucket grid -- is built
  // in buffers of its own; the context's mesh, grid and exposure-time sums
  // change only once the last step has succeeded, so every failure below
  // leaves the previous mesh in use.
  const int gstride = c->mesh.dims == 3 ? 16 : 12;
  int4* n_elem = nullptr;
  double* n_geom = nullptr;
  float* n_geo32 = nullptr;
  double4_32a* n_nodes = nullptr;
  int* n_start = nullptr;
  int* n_ids = nullptr;
  int* d_count = nullptr;
  long long* d_tmp = nullptr;
  auto drop_new = [&]() {
    cudaStreamSynchronize(c->stream);  // nothing queued may still write them
    cudaFree(n_elem);
    cudaFree(n_geom);
    cudaFree(n_geo32);
    cudaFree(n_nodes);
    cudaFree(n_start);
    cudaFree(n_ids);
    cudaFree(d_count);
    cudaFree(d_tmp);
  };
  if (cudaMalloc(&n_elem, sizeof(int4) * 2 * (size_t)nelem) != cudaSuccess ||
      cudaMalloc(&n_geom, sizeof(double) * gstride * (size_t)nelem) != cudaSuccess ||
      cudaMalloc(&n_geo32, sizeof(float) * 20 * (size_t)nelem) != cudaSuccess ||
      cudaMalloc(&n_nodes, sizeof(double4_32a) * hn.size()) != cudaSuccess) {
    drop_new();
    return fail(c, FVC_ERR_OOM, "mesh allocation failed");
  }
  // node ids and neighbours go up as given (into the geometry buffer, free
  // until the geometry kernel fills it) and are interleaved and range-checked
  // on the device, which keeps every later gather in bounds
  int4* raw = reinterpret_cast<int4*>(n_geom);
  int* d_bad = reinterpret_cast<int*>(n_geo32);
  int bad = -1;
  if (cudaMemcpyAsync(raw, conn, sizeof(int4) * (size_t)nelem, cudaMemcpyHostToDevice, c->stream) != cudaSuccess ||
      cudaMemcpyAsync(raw + nelem, adj, sizeof(int4) * (size_t)nelem, cudaMemcpyHostToDevice, c->stream) !=
          cudaSuccess ||
      cudaMemsetAsync(d_bad, 0x7f, sizeof(int), c->stream) != cudaSuccess) {
    drop_new();
    return fail(c, FVC_ERR_CUDA, "mesh upload failed");
  }
  pack_elements(raw, raw + nelem, nelem, nnodes, nv, n_elem, d_bad, c->stream);
  if (cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
      cudaStreamSynchronize(c->stream) != cudaSuccess) {
    drop_new();
    return fail(c, FVC_ERR_CUDA, "mesh check failed: %s", cudaGetErrorString(cudaGetLastError()));
  }
  if (bad < nelem) {
    drop_new();
    for (int k = 0; k < nv; k++) {
      const int nd = conn[4L * bad + k], nb = adj[4L * bad + k];
      if (nd < 0 || nd >= nnodes) return fail(c, FVC_ERR_ARG, "element %d: node %d out of range", bad, nd);
      if (nb < -1 || nb >= nelem) return fail(c, FVC_ERR_ARG, "element %d: neighbour %d out of range", bad, nb);
    }
    return fail(c, FVC_ERR_ARG, "element %d out of range", bad);
  }
  if (cudaMemcpyAsync(n_nodes, hn.data(), sizeof(double4_32a) * hn.size(), cudaMemcpyHostToDevice, c->stream) !=
      cudaSuccess) {
    drop_new();
    return fail(c, FVC_ERR_CUDA, "mesh node upload failed");
  }
  DevMesh m = c->mesh;
  m.elem = n_elem;
  m.geom = n_geom;
  m.geo32 = n_geo32;
  m.geo32lo = reinterpret_cast<const float4*>(n_geo32 + 16L * nelem);
  m.nodes = n_nodes;
  m.nelem = nelem;
  m.nnodes = nnodes;
  launch_geometry(m, n_geom, n_geo32, c->stream);
  if (cudaGetLastError() != cudaSuccess) {
    drop_new();
    return fail(c, FVC_ERR_CUDA, "geometry launch failed");
  }

  // Uniform bucket grid over the mesh's bounding box, about two elements per
  // cell, for the lowest-id global search.
  BucketGrid g = c->grid;
  int dims = m.dims;
  double ext[3], vol = 1.0;
  for (int a = 0; a < 3; a++) {
    double pad = 1e-6 * fmax(hi[a] - lo[a], 1e-300) + 1e-300;
    g.lo[a] = lo[a] - pad;
    ext[a] = (hi[a] + pad) - g.lo[a];
    if (a < dims) vol *= ext[a];
  }
  double cell = pow(vol / fmax(1.0, nelem / 2.0), 1.0 / dims);
  long ncells = 1;
  for (int a = 0; a < 3; a++) {
    if (a >= dims) {
      g.n[a] = 1;
      g.inv[a] = 0.0;
      continue;
    }
    long na = (long)ceil(ext[a] / cell);
    na = na < 1 ? 1 : (na > 4096 ? 4096 : na);
    g.n[a] = (int)na;
    g.inv[a] = (double)na / ext[a];
    ncells *= na;
  }
  const long cap = bucket_cell_cap();
  if (ncells > cap) {
    drop_new();
    return fail(c, FVC_ERR_ARG, "bucket grid too large (%ld cells, at most %ld)", ncells, cap);
  }
  if (cudaMalloc(&n_start, sizeof(int) * (ncells + 1)) != cudaSuccess ||
      cudaMalloc(&d_count, sizeof(int) * ncells) != cudaSuccess ||
      cudaMalloc(&d_tmp, sizeof(long long) * (ncells / 1024 + 8)) != cudaSuccess) {
    drop_new();
    return fail(c, FVC_ERR_OOM, "bucket grid allocation failed");
  }
  bucket_count(m, g, d_count, (int)ncells, nullptr, c->stream);
  scan_counts(d_count, n_start, (int)ncells, d_tmp, c->stream);
  int total = 0;
  if (cudaMemcpyAsync(&total, n_start + ncells, sizeof(int), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
      cudaStreamSynchronize(c->stream) != cudaSuccess) {
    drop_new();
    return fail(c, FVC_ERR_CUDA, "bucket grid count failed: %s", cudaGetErrorString(cudaGetLastError()));
  }
  if (total < 0 || cudaMalloc(&n_ids, sizeof(int) * ((size_t)total + 1)) != cudaSuccess) {
    drop_new();
    return fail(c, FVC_ERR_OOM, "bucket list allocation failed (%d entries)", total);
  }
  g.start = n_start;
  g.ids = n_ids;
  bucket_fill(m, g, n_start, d_count, n_ids, (int)ncells, nullptr, c->stream);
  if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(c->stream) != cudaSuccess) {
    drop_new();
    return fail(c, FVC_ERR_CUDA, "bucket grid build failed: %s", cudaGetErrorString(cudaGetLastError()));
  }
  cudaFree(d_count);
  cudaFree(d_tmp);

  // the new mesh is valid: it replaces the old one
  if (c->cet_sub) fvc_cet_enable(c, 0);  // the accumulators belong to the old mesh
  cudaFree(c->d_elem); c->d_elem = n_elem;
  cudaFree(c->d_geom); c->d_geom = n_geom;
  cudaFree(c->d_geo32); c->d_geo32 = n_geo32;
  cudaFree(c->d_nodes); c->d_nodes = n_nodes;
  cudaFree(c->d_cell_start); c->d_cell_start = n_start;
  cudaFree(c->d_cell_ids); c->d_cell_ids = n_ids;
  c->mesh = m;
  c->grid = g;
  for (int a = 0; a < 3; a++) {
    c->node_lo[a] = lo[a];
    c->node_hi[a] = hi[a];
  }
  if (c->frame_nodes && c->frame_nodes != nnodes) {
    for (auto& kv : c->frames) cudaFree(kv.second);
    c->frames.clear();
    drop_quantised(c);
  }
  c->frame_nodes = nnodes;
  c->mesh_set = true;
  return FVC_OK;
}

extern "C" fvc_status fvc_set_bounds(fvc_ctx* c, const double b[6]) {
  if (!c || !b) return FVC_ERR_ARG;
  for (int i = 0; i < 6; i++) c->mesh.bounds[i] = b[i];
  return FVC_OK;
}

extern "C" fvc_status fvc_set_rkf(fvc_ctx* c, double accuracy, double min_step, double max_step) {
  if (!c) return FVC_ERR_ARG;
  if (!(accuracy >= 1.0e-10) || !(min_step >= 1.0e-10) || !(max_step >= 1.0e-10))
    return fail(c, FVC_ERR_ARG, "RKF integration parameters must be positive");
  c->integ.acc = accuracy;
  c->integ.hmin = min_step;
  c->integ.hmax = max_step;
  return FVC_OK;
}

extern "C" fvc_status fvc_set_integrator(fvc_ctx* c, int int_type, double h, int extrapolate) {
  if (!c) return FVC_ERR_ARG;
  if (int_type < 0 || int_type > 3)
    return fail(c, FVC_ERR_ARG, "Int_Type %d not supported (0 Euler, 1 RK4, 2 RKF, 3 AB2)", int_type);
  if (!(h > 0) && int_type != 2) return fail(c, FVC_ERR_ARG, "Int_TimeStep must be positive");
  c->integ.type = int_type;
  c->integ.h = h;
  c->integ.extrapolate = extrapolate ? 1 : 0;
  c->integ_set = true;
  return FVC_OK;
}

// ---------------------------------------------------------------- frames

// Cartesian 2D frames whose w components are all +0.0: GetVelocity_Cartesian's
// w sum over them is exactly +0.0, so the kernels skip it.  Each of its eight
// products of +0.0 with a weight is a zero, and at least one is +0.0: a
// weight t x y, t x (1-y), ..., (1-t)(1-x)(1-y) is negative (or -0) only if
// an odd number of its factors is, and t and 1-t (x and 1-x, y and 1-y)
// cannot both be, so not all eight are; a sum of zeros holding a +0.0 is
// +0.0.  Other meshes use no flag.
static void note_wzero(fvc_ctx* c, int frame_id, const double* uvw) {
  if (c->mesh.dims != 2 || c->mesh.mesh_type != 0) return;
  bool z = true;
  for (long i = 0; i < c->frame_nodes && z; i++) {
    unsigned long long b;
    memcpy(&b, uvw + 3 * i + 2, sizeof(b));
    z = b == 0ull;
  }
  c->frame_wzero[frame_id] = z;
}

extern "C" fvc_status fvc_upload_frame(fvc_ctx* c, int frame_id, const double* uvw) {
  if (!c || !uvw) return FVC_ERR_ARG;
  if (!c->mesh_set) return fail(c, FVC_ERR_STATE, "set the mesh before uploading frames");
  if (frame_id < 0 || frame_id >= 65536) return fail(c, FVC_ERR_ARG, "frame id %d out of range", frame_id);
  fvc_status st;
  if ((st = use_device(c))) return st;
  long n = c->frame_nodes;
  if (!c->d_stage && cudaMalloc(&c->d_stage, sizeof(double) * 3 * (size_t)n) != cudaSuccess)
    return fail(c, FVC_ERR_OOM, "frame staging allocation failed");
  double4_32a*& dst = c->frames[frame_id];
  if (!dst && cudaMalloc(&dst, sizeof(double4_32a) * (size_t)n) != cudaSuccess) {
    c->frames.erase(frame_id);
    return fail(c, FVC_ERR_OOM, "frame allocation failed");
  }
  frame_dep(c, frame_id);
  FVC_CUDA(c, cudaMemcpyAsync(c->d_stage, uvw, sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice, c->stream));
  auto qf = c->qframes.find(frame_id);
  if (qf != c->qframes.end()) qf->second.fmt = 0;  // stale: quantised again when next used
  note_wzero(c, frame_id, uvw);
  pack_frame(c->d_stage, dst, n, c->stream);
  if ((st = check_launch(c, "pack_frame"))) return st;
  FVC_CUDA(c, cudaStreamSynchronize(c->stream));
  return FVC_OK;
}

static constexpr size_t POOL_LIMIT = (size_t)16 << 30;

void* pool_get(fvc_ctx* c, size_t bytes) {
  auto it = c->pool.lower_bound(bytes);
  if (it != c->pool.end() && it->first <= 2 * bytes) {
    void* p = it->second;
    c->pool_bytes -= it->first;
    c->pool.erase(it);
    return p;
  }
  void* p = nullptr;
  if (cudaMalloc(&p, bytes) != cudaSuccess) {
    // give the pool back to the device and try once more
    for (auto& kv : c->pool) cudaFree(kv.second);
    c->pool.clear();
    c->pool_bytes = 0;
    cudaGetLastError();
    if (cudaMalloc(&p, bytes) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
  }
  return p;
}

void pool_put(fvc_ctx* c, void* p, size_t bytes) {
  if (!p) return;
  if (c->pool_bytes + bytes > POOL_LIMIT) {
    cudaFree(p);
    return;
  }
  c->pool.emplace(bytes, p);
  c->pool_bytes += bytes;
}

void frame_dep(fvc_ctx* c, int id) {
  auto e = c->frame_ev.find(id);
  if (e != c->frame_ev.end()) cudaStreamWaitEvent(c->stream, e->second, 0);
}

extern "C" fvc_status fvc_host_alloc(void** p, size_t bytes) {
  if (!p) return FVC_ERR_ARG;
  *p = nullptr;
  if (cudaMallocHost(p, bytes ? bytes : 1) != cudaSuccess) {
    *p = nullptr;
    return FVC_ERR_OOM;
  }
  return FVC_OK;
}

extern "C" void fvc_host_free(void* p) {
  if (p) cudaFreeHost(p);
}

extern "C" fvc_status fvc_upload_frame_async(fvc_ctx* c, int frame_id, const double* uvw) {
  if (!c || !uvw) return FVC_ERR_ARG;
  if (!c->mesh_set) return fail(c, FVC_ERR_STATE, "set the mesh before uploading frames");
  if (frame_id < 0 || frame_id >= 65536) return fail(c, FVC_ERR_ARG, "frame id %d out of range", frame_id);
  fvc_status st;
  if ((st = use_device(c))) return st;
  const long n = c->frame_nodes;
  const size_t bytes = sizeof(double) * 3 * (size_t)n;
  if (!c->up_stream) {
    FVC_CUDA(c, cudaStreamCreateWithFlags(&c->up_stream, cudaStreamNonBlocking));
    FVC_CUDA(c, cudaEventCreateWithFlags(&c->up_after, cudaEventDisableTiming));
  }
  for (int k = 0; k < 2; k++)
    if (!c->d_up_stage[k] && cudaMalloc(&c->d_up_stage[k], bytes) != cudaSuccess)
      return fail(c, FVC_ERR_OOM, "frame staging allocation failed");
  double4_32a*& dst = c->frames[frame_id];
  if (!dst && cudaMalloc(&dst, sizeof(double4_32a) * (size_t)n) != cudaSuccess) {
    c->frames.erase(frame_id);
    return fail(c, FVC_ERR_OOM, "frame allocation failed");
  }
  cudaEvent_t& ev = c->frame_ev[frame_id];
  if (!ev) FVC_CUDA(c, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  // work already queued on the context's stream may still read the frame
  // this upload replaces
  FVC_CUDA(c, cudaEventRecord(c->up_after, c->stream));
  FVC_CUDA(c, cudaStreamWaitEvent(c->up_stream, c->up_after, 0));
  // two staging buffers: an upload reuses one after the pack that read it,
  // which the side stream orders before it
  double* stage = c->d_up_stage[c->up_k];
  c->up_k ^= 1;
  FVC_CUDA(c, cudaMemcpyAsync(stage, uvw, bytes, cudaMemcpyHostToDevice, c->up_stream));
  pack_frame(stage, dst, n, c->up_stream);
  if ((st = check_launch(c, "pack_frame"))) return st;
  auto qf = c->qframes.find(frame_id);
  if (qf != c->qframes.end()) qf->second.fmt = 0;
  note_wzero(c, frame_id, uvw);
  FVC_CUDA(c, cudaEventRecord(ev, c->up_stream));
  return FVC_OK;
}

extern "C" fvc_status fvc_frame_ready(fvc_ctx* c, int frame_id, int* ready) {
  if (!c || !ready) return FVC_ERR_ARG;
  auto e = c->frame_ev.find(frame_id);
  if (e == c->frame_ev.end()) {
    *ready = c->frames.count(frame_id) ? 1 : 0;
    return FVC_OK;
  }
  cudaError_t q = cudaEventQuery(e->second);
  if (q == cudaErrorNotReady) {
    *ready = 0;
    return FVC_OK;
  }
  if (q != cudaSuccess) return fail(c, FVC_ERR_CUDA, "frame %d upload: %s", frame_id, cudaGetErrorString(q));
  *ready = 1;
  return FVC_OK;
}

extern "C" fvc_status fvc_frame_wait(fvc_ctx* c, int frame_id) {
  if (!c) return FVC_ERR_ARG;
  auto e = c->frame_ev.find(frame_id);
  if (e == c->frame_ev.end()) return FVC_OK;
  cudaError_t q = cudaEventSynchronize(e->second);
  if (q != cudaSuccess) return fail(c, FVC_ERR_CUDA, "frame %d upload: %s", frame_id, cudaGetErrorString(q));
  return FVC_OK;
}

// The quantised copy of a resident frame in the context's 16-bit format,
// made on first use after the frame was uploaded or the format changed.
fvc_status quantised(fvc_ctx* c, int id, fvc_ctx::QFrame** out) {
  fvc_ctx::QFrame& q = c->qframes[id];
  if (q.fmt != c->prec) {
    frame_dep(c, id);
    long n = c->frame_nodes;
    if (!q.q && cudaMalloc(&q.q, sizeof(ushort4) * (size_t)n) != cudaSuccess)
      return fail(c, FVC_ERR_OOM, "quantised frame allocation failed");
    if (!c->d_qscratch && cudaMalloc(&c->d_qscratch, 4 * sizeof(unsigned)) != cudaSuccess)
      return fail(c, FVC_ERR_OOM, "quantisation scratch allocation failed");
    if (quantize_frame(c->frames[id], n, c->prec, q.q, c->d_qscratch, q.s, c->stream))
      return fail(c, FVC_ERR_CUDA, "frame quantisation failed");
    c->aux_launches += 2;
    q.fmt = c->prec;
    q.ver++;
  }
  *out = &q;
  return FVC_OK;
}

// pair records kept per window, up to this many bytes; beyond, the window's
// scratch pair is made afresh each time
static constexpr size_t QPAIR_CACHE_BYTES = (size_t)1 << 30;

static fvc_status quantised_window(fvc_ctx* c) {
  fvc_ctx::QFrame *a = nullptr, *b = nullptr;
  fvc_status st;
  if ((st = quantised(c, c->window_lo, &a)) || (st = quantised(c, c->window_hi, &b))) return st;
  DevWindow& w = c->window;
  const size_t bytes = sizeof(uint4) * (size_t)c->frame_nodes;
  auto key = std::make_pair(c->window_lo, c->window_hi);
  auto it = c->qpairs.find(key);
  if (it == c->qpairs.end() && c->qpair_bytes + bytes <= QPAIR_CACHE_BYTES) {
    fvc_ctx::QPair P;
    if (cudaMalloc(&P.q, bytes) == cudaSuccess) {
      c->qpair_bytes += bytes;
      it = c->qpairs.emplace(key, P).first;
    }
  }
  uint4* qp;
  if (it != c->qpairs.end()) {
    fvc_ctx::QPair& P = it->second;
    if (P.fmt != c->prec || P.va != a->ver || P.vb != b->ver) {
      pair_frames(a->q, b->q, c->frame_nodes, P.q, c->stream);
      c->aux_launches++;
      if ((st = check_launch(c, "pair frames"))) return st;
      P.fmt = c->prec;
      P.va = a->ver;
      P.vb = b->ver;
    }
    qp = P.q;
  } else {
    if (!c->d_qpair && cudaMalloc(&c->d_qpair, bytes) != cudaSuccess)
      return fail(c, FVC_ERR_OOM, "quantised window allocation failed");
    pair_frames(a->q, b->q, c->frame_nodes, c->d_qpair, c->stream);
    c->aux_launches++;
    if ((st = check_launch(c, "pair frames"))) return st;
    qp = c->d_qpair;
  }
  w.qp = qp;
  for (int k = 0; k < 3; k++) {
    w.qs0[k] = a->s[k];
    w.qs1[k] = b->s[k];
  }
  w.qfmt = c->prec;
  return FVC_OK;
}

extern "C" fvc_status fvc_set_precision(fvc_ctx* c, int precision) {
  if (!c) return FVC_ERR_ARG;
  if (precision != FVC_PREC_FP64 && precision != FVC_PREC_BF16 && precision != FVC_PREC_FP16)
    return fail(c, FVC_ERR_ARG, "precision %d: use FVC_PREC_FP64, FVC_PREC_BF16 or FVC_PREC_FP16", precision);
  if (precision != FVC_PREC_FP64 && c->mesh.mesh_type != 1)
    return fail(c, FVC_ERR_ARG, "the mixed-precision form needs an unstructured mesh");
  fvc_status st;
  if ((st = use_device(c))) return st;
  c->prec = precision;
  c->mesh.prec = precision;
  if (precision && c->window_set) return quantised_window(c);
  return FVC_OK;
}

// RKF needs its parameters; the mixed form runs Euler and RK4 without
// extrapolation.
fvc_status mixed_ok(fvc_ctx* c) {
  if (c->integ.type == 2 && !(c->integ.acc > 0 && c->integ.hmin > 0 && c->integ.hmax > 0))
    return fail(c, FVC_ERR_ARG, "Int_Type 2 (RKF) needs fvc_set_rkf before advecting");
  if (!c->prec) return FVC_OK;
  if (c->integ.type != 0 && c->integ.type != 1)
    return fail(c, FVC_ERR_ARG, "the mixed-precision form runs Euler (0) and RK4 (1), not Int_Type %d", c->integ.type);
  if (c->integ.extrapolate) return fail(c, FVC_ERR_ARG, "the mixed-precision form does not extrapolate");
  return FVC_OK;
}

extern "C" fvc_status fvc_set_window(fvc_ctx* c, int lo, int hi, double tmin, double tmax) {
  if (!c) return FVC_ERR_ARG;
  auto a = c->frames.find(lo), b = c->frames.find(hi);
  if (a == c->frames.end() || b == c->frames.end())
    return fail(c, FVC_ERR_STATE, "frames %d / %d are not resident", lo, hi);
  frame_dep(c, lo);
  frame_dep(c, hi);
  c->window.f0 = a->second;
  c->window.f1 = b->second;
  c->window.tmin = tmin;
  c->window.tmax = tmax;
  c->window.rspan = rcp_for_div(tmax - tmin);
  c->window.nslots = 0;
  c->window.nsteps = 0;
  {
    auto za = c->frame_wzero.find(lo), zb = c->frame_wzero.find(hi);
    c->window.wz = za != c->frame_wzero.end() && zb != c->frame_wzero.end() && za->second && zb->second;
  }
  c->window_set = true;
  c->window_lo = lo;
  c->window_hi = hi;
  return c->prec ? quantised_window(c) : FVC_OK;
}

// The stage times of an advection call from t1 to t2, computed with the
// integrators' own arithmetic (ompVC/integration.c:345-352, 402), and, on an
// unstructured mesh, the node velocities at each of them.  A slot is only a
// hint: the kernels compare its time with the time they compute before using
// it, so the table can end early (slot cap, tloc out of range) without
// changing any result.
static fvc_status build_steps(fvc_ctx* c, double t1, double t2);

static fvc_status prepare_slots(fvc_ctx* c, double t1, double t2) {
  if (c->prec) return build_steps(c, t1, t2);
  DevWindow& w = c->window;
  w.nslots = 0;
  int n = 0;
  auto add = [&](double tq) {
    if (n >= FVC_MAX_SLOTS) return false;
    double tloc = (tq - w.tmin) / (w.tmax - w.tmin);
    if ((tloc > 1 + 1.0e-10) || (tloc < 0 - 1.0e-10)) return false;
    w.tq[n] = tq;
    w.tl[n] = tloc;
    n++;
    return true;
  };
  double tc = t1, h = (t2 - t1) >= 0.0 ? fabs(c->integ.h) : -fabs(c->integ.h);
  bool ok = true;
  while ((tc - t2) * (t2 - t1) < 0.0) {
    if ((tc + h - t2) * (tc + h - t1) > 0.0) h = (t2 - t1) >= 0.0 ? fabs(t2 - tc) : -fabs(t2 - tc);
    if (!add(tc) || !add(tc + h / 2)) {
      ok = false;
      break;
    }
    tc = tc + h;
  }
  if (ok) add(tc);
  w.nslots = n;
  if (c->mesh.mesh_type != 1 || n == 0) return FVC_OK;
  if (n > c->vt_slots) {
    cudaFree(c->d_vt);
    c->d_vt = nullptr;
    c->vt_slots = 0;
    if (cudaMalloc(&c->d_vt, sizeof(double4_32a) * (size_t)n * (size_t)c->mesh.nnodes) != cudaSuccess) {
      w.nslots = 0;  // run without the table
      return FVC_OK;
    }
    c->vt_slots = n;
  }
  w.vt = c->d_vt;
  w.vt_stride = c->mesh.nnodes;
  time_fields(c->mesh, w, c->d_vt, c->stream);
  c->aux_launches++;
  return check_launch(c, "time fields");
}

// The mixed form's step table for a call from t1 to t2: the stage times of
// the FP64 step loop (ompVC/integration.c:345-352, 402, the same sequence as
// prepare_slots), each step's length and the tloc of its stages.  A stage
// time outside the window gives FVC_ERR_TLOC for the call.
static fvc_status build_steps(fvc_ctx* c, double t1, double t2) {
  DevWindow& w = c->window;
  std::vector<StepM>& T = c->h_steps;
  T.clear();
  auto tloc = [&](double tq, float& out) {
    double tl = (tq - w.tmin) / (w.tmax - w.tmin);
    if ((tl > 1 + 1.0e-10) || (tl < 0 - 1.0e-10)) return false;
    out = (float)tl;
    return true;
  };
  double tc = t1, h = (t2 - t1) >= 0.0 ? fabs(c->integ.h) : -fabs(c->integ.h);
  while ((tc - t2) * (t2 - t1) < 0.0) {
    if ((tc + h - t2) * (tc + h - t1) > 0.0) h = (t2 - t1) >= 0.0 ? fabs(t2 - tc) : -fabs(t2 - tc);
    StepM s{};
    s.tc = tc;
    s.h = (float)h;
    if (!tloc(tc, s.tl0) || !tloc(tc + h / 2, s.tlh) || !tloc(tc + h, s.tl1))
      return fail(c, FVC_ERR_TLOC, "advect: query time outside the loaded frame interval");
    T.push_back(s);
    tc = tc + h;
  }
  StepM e{};
  e.tc = tc;
  T.push_back(e);
  constexpr int RING = 64, RING_STEPS = 128;
  if (T.size() <= (size_t)RING_STEPS) {
    if (!c->h_ring) {
      if (cudaMallocHost(&c->h_ring, sizeof(StepM) * RING * RING_STEPS) != cudaSuccess ||
          cudaMalloc(&c->d_ring, sizeof(StepM) * RING * RING_STEPS) != cudaSuccess) {
        cudaFreeHost(c->h_ring);
        c->h_ring = nullptr;
        return fail(c, FVC_ERR_OOM, "step table ring allocation failed");
      }
      c->ring_ev.assign(RING, nullptr);
      for (auto& ev : c->ring_ev) FVC_CUDA(c, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    }
    const int k = c->ring_k;
    c->ring_k = (c->ring_k + 1) % RING;
    FVC_CUDA(c, cudaEventSynchronize(c->ring_ev[k]));
    StepM* h = c->h_ring + (size_t)k * RING_STEPS;
    StepM* d = c->d_ring + (size_t)k * RING_STEPS;
    memcpy(h, T.data(), sizeof(StepM) * T.size());
    FVC_CUDA(c, cudaMemcpyAsync(d, h, sizeof(StepM) * T.size(), cudaMemcpyHostToDevice, c->stream));
    FVC_CUDA(c, cudaEventRecord(c->ring_ev[k], c->stream));
    w.steps = d;
    w.nsteps = (int)T.size() - 1;
    w.nslots = 0;
    return FVC_OK;
  }
  if (T.size() > c->steps_cap) {
    cudaFree(c->d_steps);
    c->d_steps = nullptr;
    c->steps_cap = 0;
    size_t cap = T.size() < 64 ? 64 : 2 * T.size();
    if (cudaMalloc(&c->d_steps, sizeof(StepM) * cap) != cudaSuccess)
      return fail(c, FVC_ERR_OOM, "step table allocation failed");
    c->steps_cap = cap;
  }
  FVC_CUDA(c, cudaMemcpyAsync(c->d_steps, T.data(), sizeof(StepM) * T.size(), cudaMemcpyHostToDevice, c->stream));
  w.steps = c->d_steps;
  w.nsteps = (int)T.size() - 1;
  w.nslots = 0;
  return FVC_OK;
}

static fvc_status ready(fvc_ctx* c, bool need_window) {
  if (!c) return FVC_ERR_ARG;
  if (!c->mesh_set) return fail(c, FVC_ERR_STATE, "mesh not set");
  if (need_window && !c->window_set) return fail(c, FVC_ERR_STATE, "frame window not set");
  return use_device(c);
}

// ---------------------------------------------------------------- step level

extern "C" fvc_status fvc_advect_device(fvc_ctx* c, int n, double* dX, double* dV, int* deid,
                                        int* dleft, double* dldt, double t0, double t1, long long* steps) {
  fvc_status st;
  if ((st = ready(c, true))) return st;
  if (n < 0 || (n > 0 && (!dX || !dleft || !dldt))) return fail(c, FVC_ERR_ARG, "bad arrays");
  if (c->mesh.mesh_type == 1 && n > 0 && !deid) return fail(c, FVC_ERR_ARG, "unstructured advection needs element ids");
  if (c->integ.extrapolate && n > 0 && !dV) return fail(c, FVC_ERR_ARG, "extrapolation needs V");
  if ((st = mixed_ok(c))) return st;
  if ((st = prepare_slots(c, t0, t1))) return st;
  launch_advect(c->mesh, c->window, c->integ, n, dX, dV, deid, dleft, dldt, t0, t1, c->d_ctr, c->stream);
  if ((st = check_launch(c, "advect"))) return st;
  return finish(c, "advect", steps);
}

extern "C" fvc_status fvc_advect(fvc_ctx* c, int n, double* X, double* V, int* eid, int* left,
                                 double* ldt, double t0, double t1, long long* steps) {
  fvc_status st;
  if ((st = ready(c, true))) return st;
  if (n < 0 || (n > 0 && (!X || !left || !ldt))) return fail(c, FVC_ERR_ARG, "bad arrays");
  if (steps) *steps = 0;
  if (n == 0) return FVC_OK;
  size_t bx = al256(sizeof(double) * 3 * (size_t)n), bi = al256(sizeof(int) * (size_t)n),
         bd = al256(sizeof(double) * (size_t)n);
  if ((st = ensure_scratch(c, 2 * bx + 2 * bi + bd))) return st;
  char* p = (char*)c->d_scratch;
  double* dX = (double*)p; p += bx;
  double* dV = (double*)p; p += bx;
  int* de = (int*)p; p += bi;
  int* dl = (int*)p; p += bi;
  double* dt = (double*)p;
  cudaStream_t s = c->stream;
  FVC_CUDA(c, cudaMemcpyAsync(dX, X, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s));
  if (V) FVC_CUDA(c, cudaMemcpyAsync(dV, V, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s));
  if (eid) FVC_CUDA(c, cudaMemcpyAsync(de, eid, sizeof(int) * n, cudaMemcpyHostToDevice, s));
  FVC_CUDA(c, cudaMemcpyAsync(dl, left, sizeof(int) * n, cudaMemcpyHostToDevice, s));
  FVC_CUDA(c, cudaMemcpyAsync(dt, ldt, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  if (c->mesh.mesh_type == 1 && !eid) return fail(c, FVC_ERR_ARG, "unstructured advection needs element ids");
  if (c->integ.extrapolate && !V) return fail(c, FVC_ERR_ARG, "extrapolation needs V");
  if ((st = mixed_ok(c))) return st;
  if ((st = prepare_slots(c, t0, t1))) return st;
  launch_advect(c->mesh, c->window, c->integ, n, dX, V ? dV : nullptr, eid ? de : nullptr, dl, dt, t0,
                t1, c->d_ctr, s);
  if ((st = check_launch(c, "advect"))) return st;
  FVC_CUDA(c, cudaMemcpyAsync(X, dX, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, s));
  if (V) FVC_CUDA(c, cudaMemcpyAsync(V, dV, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, s));
  if (eid) FVC_CUDA(c, cudaMemcpyAsync(eid, de, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
  FVC_CUDA(c, cudaMemcpyAsync(left, dl, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
  FVC_CUDA(c, cudaMemcpyAsync(ldt, dt, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  return finish(c, "advect", steps);
}

extern "C" fvc_status fvc_velocity(fvc_ctx* c, int n, const double* X, int* eid, int* left, double tq,
                                   double* out) {
  fvc_status st;
  if ((st = ready(c, true))) return st;
  if (n < 0 || (n > 0 && (!X || !left || !out))) return fail(c, FVC_ERR_ARG, "bad arrays");
  if (c->mesh.mesh_type == 1 && n > 0 && !eid) return fail(c, FVC_ERR_ARG, "unstructured velocity needs element ids");
  if (n == 0) return FVC_OK;
  size_t bx = al256(sizeof(double) * 3 * (size_t)n), bi = al256(sizeof(int) * (size_t)n);
  if ((st = ensure_scratch(c, 2 * bx + 2 * bi))) return st;
  char* p = (char*)c->d_scratch;
  double* dX = (double*)p; p += bx;
  double* dO = (double*)p; p += bx;
  int* de = (int*)p; p += bi;
  int* dl = (int*)p;
  cudaStream_t s = c->stream;
  FVC_CUDA(c, cudaMemcpyAsync(dX, X, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s));
  if (eid) FVC_CUDA(c, cudaMemcpyAsync(de, eid, sizeof(int) * n, cudaMemcpyHostToDevice, s));
  FVC_CUDA(c, cudaMemcpyAsync(dl, left, sizeof(int) * n, cudaMemcpyHostToDevice, s));
  launch_velocity(c->mesh, c->window, n, dX, eid ? de : nullptr, dl, tq, dO, c->d_ctr, s);
  if ((st = check_launch(c, "velocity"))) return st;
  FVC_CUDA(c, cudaMemcpyAsync(out, dO, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, s));
  if (eid) FVC_CUDA(c, cudaMemcpyAsync(eid, de, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
  FVC_CUDA(c, cudaMemcpyAsync(left, dl, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
  return finish(c, "velocity", nullptr);
}

extern "C" fvc_status fvc_local_search(fvc_ctx* c, int n, const double* X, const int* guess, int* out) {
  fvc_status st;
  if ((st = ready(c, false))) return st;
  if (c->mesh.mesh_type != 1) return fail(c, FVC_ERR_STATE, "local search needs an unstructured mesh");
  if (n < 0 || (n > 0 && (!X || !guess || !out))) return fail(c, FVC_ERR_ARG, "bad arrays");
  if (n == 0) return FVC_OK;
  size_t bx = al256(sizeof(double) * 3 * (size_t)n), bi = al256(sizeof(int) * (size_t)n);
  if ((st = ensure_scratch(c, bx + 2 * bi))) return st;
  char* p = (char*)c->d_scratch;
  double* dX = (double*)p; p += bx;
  int* dg = (int*)p; p += bi;
  int* dO = (int*)p;
  cudaStream_t s = c->stream;
  FVC_CUDA(c, cudaMemcpyAsync(dX, X, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s));
  FVC_CUDA(c, cudaMemcpyAsync(dg, guess, sizeof(int) * n, cudaMemcpyHostToDevice, s));
  launch_local_search(c->mesh, n, dX, dg, dO, c->d_ctr, s);
  if ((st = check_launch(c, "local search"))) return st;
  FVC_CUDA(c, cudaMemcpyAsync(out, dO, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
  return finish(c, "local search", nullptr);
}

extern "C" fvc_status fvc_global_search(fvc_ctx* c, int n, const double* X, int* out) {
  fvc_status st;
  if ((st = ready(c, false))) return st;
  if (c->mesh.mesh_type != 1) return fail(c, FVC_ERR_STATE, "global search needs an unstructured mesh");
  if (n < 0 || (n > 0 && (!X || !out))) return fail(c, FVC_ERR_ARG, "bad arrays");
  if (n == 0) return FVC_OK;
  size_t bx = al256(sizeof(double) * 3 * (size_t)n), bi = al256(sizeof(int) * (size_t)n);
  if ((st = ensure_scratch(c, bx + bi))) return st;
  char* p = (char*)c->d_scratch;
  double* dX = (double*)p; p += bx;
  int* dO = (int*)p;
  cudaStream_t s = c->stream;
  FVC_CUDA(c, cudaMemcpyAsync(dX, X, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s));
  launch_global_search(c->mesh, c->grid, n, dX, nullptr, dO, s);
  if ((st = check_launch(c, "global search"))) return st;
  FVC_CUDA(c, cudaMemcpyAsync(out, dO, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
  return finish(c, "global search", nullptr);
}

// ---------------------------------------------------------------- jobs

// Frees a job that no queued GPU work uses any more (its last kernels have
// completed and nothing reads it on another stream): as fvc_job_destroy,
// without waiting for the context's stream.
void job_destroy_idle(fvc_job* j) {
  if (!j) return;
  if (j->ctx) {
    cudaSetDevice(j->ctx->device);
    pool_put(j->ctx, j->mem, j->mem_bytes);
    pool_put(j->ctx, j->rec_mem, j->rec_bytes);
  } else {
    cudaFree(j->mem);
    cudaFree(j->rec_mem);
  }
  if (j->d_ctr) cudaFree(j->d_ctr);
  for (int k = 0; k < 4; k++)
    if (j->ev[k]) cudaEventDestroy(j->ev[k]);
  for (cudaEvent_t e : j->pend) cudaEventDestroy(e);
  for (cudaEvent_t e : j->spare) cudaEventDestroy(e);
  delete j;
}

extern "C" void fvc_job_destroy(fvc_job* j) {
  if (!j) return;
  if (j->ctx) {
    cudaSetDevice(j->ctx->device);
    cudaStreamSynchronize(j->ctx->stream);
  }
  if (j->ctx) {
    pool_put(j->ctx, j->mem, j->mem_bytes);
    pool_put(j->ctx, j->rec_mem, j->rec_bytes);
  } else {
    cudaFree(j->mem);
    cudaFree(j->rec_mem);
  }
  cudaFree(j->d_ctr);
  for (int k = 0; k < 4; k++)
    if (j->ev[k]) cudaEventDestroy(j->ev[k]);
  for (cudaEvent_t e : j->pend) cudaEventDestroy(e);
  for (cudaEvent_t e : j->spare) cudaEventDestroy(e);
  delete j;
}

// Waits for the job's asynchronous FTLE intervals and accounts them: steps
// and device times into the stats, fault bits into the returned status.
static fvc_status job_sync(fvc_job* j, const char* what) {
  if (!j->d_ctr) return FVC_OK;
  fvc_ctx* c = j->ctx;
  DevCounters h{};
  FVC_CUDA(c, cudaMemcpyAsync(&h, j->d_ctr, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  FVC_CUDA(c, cudaStreamSynchronize(c->stream));
  // only the accumulated counts and the fault bits are taken: the live
  // lists' counts and cursors stay for the job's next call
  FVC_CUDA(c, cudaMemsetAsync(j->d_ctr, 0, offsetof(DevCounters, changed) + sizeof(int), c->stream));
  FVC_CUDA(c, cudaMemsetAsync(&j->d_ctr->steps_rec, 0, sizeof(j->d_ctr->steps_rec), c->stream));
  j->stats.steps_main += (long long)h.steps;
  j->stats.steps_early += (long long)h.steps_early;
  j->stats.steps_early_recorded += (long long)h.steps_rec;
  for (size_t k = 0; k + 2 < j->pend.size(); k += 3) {
    j->stats.ms_main += ev_ms(j->pend[k], j->pend[k + 1]);
    j->stats.ms_early += ev_ms(j->pend[k + 1], j->pend[k + 2]);
  }
  j->spare.insert(j->spare.end(), j->pend.begin(), j->pend.end());
  j->pend.clear();
  if (h.status & PT_ERR_STATE)
    return fail(c, FVC_ERR_STATE, "%s: a point that had left the domain was advected", what);
  if (h.status & PT_ERR_TLOC)
    return fail(c, FVC_ERR_TLOC, "%s: query time outside the loaded frame interval", what);
  if (h.status & PT_ERR_WALK)
    return fail(c, FVC_ERR_WALK, "%s: neighbour walk failed (indeterminate neighbour or hop cap)", what);
  if (h.status & PT_ERR_CET)
    return fail(c, FVC_ERR_WALK, "%s: exposure time: a step started outside the velocity domain", what);
  return FVC_OK;
}

extern "C" fvc_status fvc_job_get_stats(fvc_job* j, fvc_job_stats* out) {
  if (!j || !out) return FVC_ERR_ARG;
  fvc_status st = FVC_OK;
  if (j->d_ctr && use_device(j->ctx) == FVC_OK) st = job_sync(j, j->kind == 1 ? "tracer advance" : "ftle interval");
  *out = j->stats;
  return st;
}

extern "C" void* fvc_stream(fvc_ctx* c) { return c ? (void*)c->stream : nullptr; }

// Carves one allocation into the arrays listed in sizes (bytes each).
static fvc_status carve(fvc_ctx* c, void** mem, std::vector<std::pair<void**, size_t>> parts,
                        size_t* bytes = nullptr) {
  size_t total = 0;
  for (auto& p : parts) total += al256(p.second);
  if (!total) total = 256;
  *mem = pool_get(c, total);
  if (!*mem) return fail(c, FVC_ERR_OOM, "could not allocate %zu bytes for the job", total);
  if (bytes) *bytes = total;
  char* q = (char*)*mem;
  for (auto& p : parts) {
    *p.first = q;
    q += al256(p.second);
  }
  return FVC_OK;
}

static fvc_status run_chain(fvc_ctx* c, const ChainArgs& a, const double* dX, const int* dleft0, int* deid,
                            long long* launches) {
  const size_t words = chain_words(a);
  int* work = (int*)pool_get(c, sizeof(int) * words);
  if (!work) return fail(c, FVC_ERR_OOM, "seed-chain scratch");
  int rounds = locate_chain(c->mesh, c->grid, a, dX, dleft0, deid, work, c->d_ctr, c->stream);
  cudaStreamSynchronize(c->stream);
  pool_put(c, work, sizeof(int) * words);
  if (rounds < 0) {
    fvc_status st = finish(c, "seed location", nullptr);
    return st ? st : fail(c, FVC_ERR_CUDA, "seed location failed");
  }
  // the three-level FTLE chain (rounds == 0), or the global search +
  // first-found and per round the guess kernels and the walk
  *launches += rounds == 0 ? 3 : 2 + (long long)rounds * (a.kind == 0 ? 6 : 4);
  return FVC_OK;
}

static int center_element(fvc_ctx* c, const double X[3]) {
  int r = -1;
  char* buf = (char*)pool_get(c, 256);
  if (!buf) return -2;
  double* dX = (double*)buf;
  int* dO = (int*)(buf + 64);
  cudaMemcpyAsync(dX, X, 3 * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  launch_global_search(c->mesh, c->grid, 1, dX, nullptr, dO, c->stream);
  cudaMemcpyAsync(&r, dO, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) r = -2;
  pool_put(c, buf, 256);
  return r;
}

extern "C" fvc_status fvc_ftle_create(fvc_ctx* c, const fvc_ftle_spec* sp, fvc_job** out) {
  fvc_status st;
  if (!out || !sp) return fail(c, FVC_ERR_ARG, "null argument");
  *out = nullptr;
  if ((st = ready(c, false))) return st;
  int dims = c->mesh.dims;
  int xr = sp->xres, yr = sp->yres, zr = dims == 3 ? sp->zres : 1;
  if (xr < 2 || yr < 2 || (dims == 3 && zr < 2) || zr < 1) return fail(c, FVC_ERR_ARG, "FTLE grid resolution too small");
  long n = (long)xr * yr * zr;
  if (n > (1L << 30)) return fail(c, FVC_ERR_ARG, "FTLE grid too large");
  fvc_job* j = new fvc_job();
  j->ctx = c;
  j->kind = 0;
  FtleDev& f = j->f;
  f.n = (int)n;
  f.xr = xr;
  f.yr = yr;
  f.zr = zr;
  // FTLE_CartMesh deltas, ompVC/parameters.c:311-320
  f.dx = (sp->xmax - sp->xmin) / (xr - 1);
  f.dy = (sp->ymax - sp->ymin) / (yr - 1);
  f.dz = dims == 3 ? (sp->zmax - sp->zmin) / (zr - 1) : 0.0;
  f.start = sp->start_time;
  f.mixed = c->prec ? 1 : 0;
  j->prec = c->prec;
  int* left0 = nullptr;
  st = carve(c, &j->mem,
             {{(void**)&f.X, 24 * n}, {(void**)&f.V, 24 * n}, {(void**)&f.ldt, 8 * n}, {(void**)&f.ftT, 8 * n},
              {(void**)&f.ftN, 8 * n}, {(void**)&f.eid, 4 * n}, {(void**)&f.left, 4 * n}, {(void**)&f.have, 4 * n},
              {(void**)&f.Xn, 24 * n}, {(void**)&f.Vn, 24 * n}, {(void**)&f.te, 8 * n}, {(void**)&f.en, 4 * n},
              {(void**)&f.flag, n}, {(void**)&f.served, 4 * n}, {(void**)&f.trig, 4 * n}, {(void**)&f.out, 16 * n},
              {(void**)&f.epos, 168 * n}, {(void**)&f.elt, 48 * n}, {(void**)&f.emt, 8 * n},
              {(void**)&f.tasks, 56 * n}, {(void**)&f.tsorted, 56 * n}, {(void**)&f.live, 4 * n},
              {(void**)&f.block_cnt, sizeof(int) * (2 * (n / 1024 + 1) + 16) + sizeof(long long) * (n / 1048576 + 8)},
              {(void**)&left0, 4 * n}},
             &j->mem_bytes);
  if (st) {
    delete j;
    return st;
  }
  job_events(j);
  cudaEventRecord(j->ev[3], c->stream);
  if (sp->generate) {
    double zmin = dims == 3 ? sp->zmin : 0.0;
    ftle_seed_grid(c->mesh, f, sp->xmin, sp->ymin, zmin, left0, c->stream);
    if ((st = check_launch(c, "ftle seed"))) { fvc_job_destroy(j); return st; }
    if (c->mesh.mesh_type == 1) {
      // centre seed, ompVC/ftle.c:457-465
      double Xs[3] = {sp->xmin + ((int)(xr / 2)) * f.dx, sp->ymin + ((int)(yr / 2)) * f.dy,
                      zmin + ((int)(zr / 2)) * f.dz};
      int center = center_element(c, Xs);
      if (center < -1) { fvc_job_destroy(j); return fail(c, FVC_ERR_CUDA, "centre search failed"); }
      ChainArgs a{0, (int)n, {xr, yr, zr}, sp->local_search_checking, center};
      j->stats.launches += 1;
      if ((st = run_chain(c, a, f.X, left0, f.eid, &j->stats.launches))) { fvc_job_destroy(j); return st; }
    }
    ftle_init_marks(c->mesh, f, left0, c->stream);
    ftle_mark_outside(f, c->stream);
    j->stats.launches += 3;
    if ((st = check_launch(c, "ftle marks"))) { fvc_job_destroy(j); return st; }
  }
  if (j->prec) {
    pack_pairs(f.X, 3 * n, c->stream);
    j->packed = true;
  }
  cudaEventRecord(j->ev[0], c->stream);
  FVC_CUDA(c, cudaStreamSynchronize(c->stream));
  j->stats.ms_setup += ev_ms(j->ev[3], j->ev[0]);
  *out = j;
  return FVC_OK;
}

extern "C" fvc_status fvc_ftle_set_state(fvc_job* j, const double* X, const int* eid, const int* left,
                                         const double* ldt, const int* have, const double* wT, const double* wN) {
  if (!j || j->kind != 0) return FVC_ERR_ARG;
  fvc_ctx* c = j->ctx;
  fvc_status st;
  if ((st = use_device(c))) return st;
  if ((st = job_sync(j, "ftle interval"))) return st;
  FtleDev& f = j->f;
  size_t n = (size_t)f.n;
  cudaStream_t s = c->stream;
  j->live_ready = false;  // the next interval compacts the live points afresh
  if (X) {
    FVC_CUDA(c, cudaMemcpyAsync(f.X, X, 24 * n, cudaMemcpyHostToDevice, s));
    if (j->packed) pack_pairs(f.X, 3 * (long)n, s);
  }
  if (eid) {
    std::vector<int> chk(eid, eid + n);
    for (size_t i = 0; i < n; i++)
      if (chk[i] >= c->mesh.nelem && c->mesh.mesh_type == 1) return fail(c, FVC_ERR_ARG, "element id out of range");
    FVC_CUDA(c, cudaMemcpyAsync(f.eid, eid, 4 * n, cudaMemcpyHostToDevice, s));
  }
  if (left) FVC_CUDA(c, cudaMemcpyAsync(f.left, left, 4 * n, cudaMemcpyHostToDevice, s));
  if (ldt) FVC_CUDA(c, cudaMemcpyAsync(f.ldt, ldt, 8 * n, cudaMemcpyHostToDevice, s));
  if (have) FVC_CUDA(c, cudaMemcpyAsync(f.have, have, 4 * n, cudaMemcpyHostToDevice, s));
  if (wT) FVC_CUDA(c, cudaMemcpyAsync(f.ftT, wT, 8 * n, cudaMemcpyHostToDevice, s));
  if (wN) FVC_CUDA(c, cudaMemcpyAsync(f.ftN, wN, 8 * n, cudaMemcpyHostToDevice, s));
  FVC_CUDA(c, cudaMemsetAsync(f.V, 0, 24 * n, s));
  FVC_CUDA(c, cudaStreamSynchronize(s));
  return FVC_OK;
}

extern "C" fvc_status fvc_ftle_get_state(fvc_job* j, double* X, int* eid, int* left, double* ldt, int* have,
                                         double* wT, double* wN) {
  if (!j || j->kind != 0) return FVC_ERR_ARG;
  fvc_ctx* c = j->ctx;
  fvc_status st;
  if ((st = use_device(c))) return st;
  if ((st = job_sync(j, "ftle interval"))) return st;
  FtleDev& f = j->f;
  size_t n = (size_t)f.n;
  cudaStream_t s = c->stream;
  if (X) FVC_CUDA(c, cudaMemcpyAsync(X, f.X, 24 * n, cudaMemcpyDeviceToHost, s));
  if (eid) FVC_CUDA(c, cudaMemcpyAsync(eid, f.eid, 4 * n, cudaMemcpyDeviceToHost, s));
  if (left) FVC_CUDA(c, cudaMemcpyAsync(left, f.left, 4 * n, cudaMemcpyDeviceToHost, s));
  if (ldt) FVC_CUDA(c, cudaMemcpyAsync(ldt, f.ldt, 8 * n, cudaMemcpyDeviceToHost, s));
  if (have) FVC_CUDA(c, cudaMemcpyAsync(have, f.have, 4 * n, cudaMemcpyDeviceToHost, s));
  if (wT) FVC_CUDA(c, cudaMemcpyAsync(wT, f.ftT, 8 * n, cudaMemcpyDeviceToHost, s));
  if (wN) FVC_CUDA(c, cudaMemcpyAsync(wN, f.ftN, 8 * n, cudaMemcpyDeviceToHost, s));
  FVC_CUDA(c, cudaStreamSynchronize(s));
  if (X && j->packed) unpack_host(X, 3 * n);
  return FVC_OK;
}

extern "C" fvc_status fvc_ftle_interval(fvc_job* j, int launch, double t1, double t2, long long* steps) {
  if (!j || j->kind != 0) return FVC_ERR_ARG;
  fvc_ctx* c = j->ctx;
  fvc_status st;
  if ((st = ready(c, true))) return st;
  cudaStream_t s = c->stream;
  job_events(j);
  if (j->prec != c->prec) return fail(c, FVC_ERR_STATE, "the job was created with another precision form");
  if ((st = mixed_ok(c))) return st;
  if (j->prec && !j->packed) {
    pack_pairs(j->f.X, 3L * j->f.n, s);
    j->packed = true;
    j->stats.launches++;
  }
  if ((st = prepare_slots(c, t1, t2))) return st;
  // the main pass's per-step record, from which early-FTLE advections that
  // repeat it are read (Euler and RK4 with a fixed step sequence)
  j->f.rec = nullptr;
  j->f.kacc = nullptr;
  j->f.rec_e1 = nullptr;
  j->f.rec_steps = 0;
  if ((c->integ.type == 0 || c->integ.type == 1) && !c->integ.extrapolate) {
    const int ns = j->prec ? c->window.nsteps : (c->window.nslots > 0 ? (c->window.nslots - 1) / 2 : 0);
    const int want = ns < 32 ? ns : 32;
    if (want > 0 && want > j->rec_cap) {
      pool_put(c, j->rec_mem, j->rec_bytes);
      j->rec_mem = nullptr;
      j->rec_cap = 0;
      const size_t n = (size_t)j->f.n;
      // positions, accepted steps, step-1 element states
      j->rec_bytes = al256(24 * n * (size_t)want) + al256(n) + 16 * n;
      j->rec_mem = pool_get(c, j->rec_bytes);
      if (j->rec_mem) j->rec_cap = want;
    }
    if (want > 0 && j->rec_cap >= want) {
      j->f.rec = (double*)j->rec_mem;
      const size_t n = (size_t)j->f.n, pos_bytes = al256(24 * n * (size_t)j->rec_cap);
      j->f.kacc = (unsigned char*)j->rec_mem + pos_bytes;
      if (!j->prec && c->integ.type == 1) j->f.rec_e1 = (int4*)((char*)j->rec_mem + pos_bytes + al256(n));
      j->f.rec_steps = want;
    }
  }
  if (!j->d_ctr) {
    if (cudaMalloc(&j->d_ctr, sizeof(DevCounters)) != cudaSuccess) return fail(c, FVC_ERR_OOM, "job counters");
    FVC_CUDA(c, cudaMemsetAsync(j->d_ctr, 0, sizeof(DevCounters), s));
  }
  DevCounters* ctr = j->d_ctr;
  cudaEvent_t ev[3];
  for (int k = 0; k < 3; k++) {
    if (!j->spare.empty()) {
      ev[k] = j->spare.back();
      j->spare.pop_back();
    } else if (cudaEventCreate(&ev[k]) != cudaSuccess) {
      return fail(c, FVC_ERR_CUDA, "event creation failed");
    }
    j->pend.push_back(ev[k]);
  }
  // the persistent launches' work cursors start at 0 every interval: the
  // live-list kernels (ftle_live, or the previous interval's update) clear
  // them, and the main pass clears the early-FTLE counters
  if (launch) ftle_launch(c->mesh, c->window, j->f, j->f.start, ctr, s);
  // the previous interval's update built the live list, unless the state
  // was set from the host since
  const bool compact = launch || !j->live_ready;
  if (compact) ftle_live(c->integ, j->f, ctr, s);
  cudaEventRecord(ev[0], s);
  ftle_pass1(c->mesh, c->window, c->integ, j->f, t1, t2, ctr, s);
  cudaEventRecord(ev[1], s);
  if (!c->integ.extrapolate) {
    ftle_triggers(j->f, ctr, true, s);
    ftle_early(c->mesh, c->window, c->integ, j->f, t1, ctr, false, s);
  }
  cudaEventRecord(ev[2], s);
  ftle_update(c->mesh, c->integ, j->f, ctr, s);
  j->live_ready = true;
  if ((st = check_launch(c, "ftle interval"))) return st;
  j->stats.intervals++;
  // launch, the live list, the main pass,
  // triggers and the early-FTLE kernels, the update
  j->stats.launches += (launch ? 1 : 0) + (compact ? 1 : 0) + 1 +
                       (c->integ.extrapolate ? 0 : 1 + (j->prec ? 5 : 7)) + 1 + c->aux_launches;
  c->aux_launches = 0;
  if (!steps) return FVC_OK;  // asynchronous: accounted by the next call that waits
  const long long before = j->stats.steps_main + j->stats.steps_early;
  st = job_sync(j, "ftle interval");
  *steps = j->stats.steps_main + j->stats.steps_early - before;
  return st;
}

extern "C" fvc_status fvc_ftle_reduce(fvc_job* j, double int_t, double* wT, double* wN) {
  if (!j || j->kind != 0) return FVC_ERR_ARG;
  fvc_ctx* c = j->ctx;
  fvc_status st;
  if ((st = use_device(c))) return st;
  if ((st = job_sync(j, "ftle interval"))) return st;
  job_events(j);
  if (j->packed) {
    unpack_pairs(j->f.X, 3L * j->f.n, c->stream);
    j->packed = false;
    j->stats.launches++;
  }
  cudaEventRecord(j->ev[0], c->stream);
  ftle_final(j->f, c->mesh.dims, int_t, c->stream);
  cudaEventRecord(j->ev[1], c->stream);
  if ((st = check_launch(c, "ftle reduce"))) return st;
  size_t n = (size_t)j->f.n;
  if (wT) FVC_CUDA(c, cudaMemcpyAsync(wT, j->f.out, 8 * n, cudaMemcpyDeviceToHost, c->stream));
  if (wN) FVC_CUDA(c, cudaMemcpyAsync(wN, j->f.out + n, 8 * n, cudaMemcpyDeviceToHost, c->stream));
  FVC_CUDA(c, cudaStreamSynchronize(c->stream));
  j->stats.ms_reduce += ev_ms(j->ev[0], j->ev[1]);
  j->stats.launches += 1;
  return FVC_OK;
}

// ------------------------------------------------ exposure / residence time

static CetDev cet_dev(const fvc_ctx* c) {
  CetDev d{};
  d.sum = c->d_cet_sum;
  d.enc = c->d_cet_enc;
  d.substeps = c->cet_sub;
  d.g = c->grid;
  return d;
}

// Exposure time runs in the FP64 form with Euler, RK4 or RKF, as ompVC's
// integrators call ComputeExposureTime (integration.c:183-203, 277-299,
// 427-447, 649-669); ompVC has no multistep integrator.
static fvc_status cet_ok(fvc_ctx* c, const fvc_job* j) {
  if (!c->cet_sub) return FVC_OK;
  if (j->prec) return fail(c, FVC_ERR_ARG, "exposure time is computed in the FP64 form only");
  if (c->integ.type == 3) return fail(c, FVC_ERR_ARG, "exposure time needs Int_Type 0, 1 or 2");
  return FVC_OK;
}

extern "C" fvc_status fvc_cet_enable(fvc_ctx* c, int substeps) {
  if (!c) return FVC_ERR_ARG;
  fvc_status st;
  if ((st = use_device(c))) return st;
  if (substeps == 0) {
    cudaFree(c->d_cet_sum);
    cudaFree(c->d_cet_enc);
    c->d_cet_sum = nullptr;
    c->d_cet_enc = nullptr;
    c->cet_sub = 0;
    return FVC_OK;
  }
  if (substeps < 2) return fail(c, FVC_ERR_ARG, "Trace_CETSubsteps must be greater than 1");
  if (c->mesh.mesh_type != 1 || !c->mesh_set)
    return fail(c, FVC_ERR_STATE, "exposure time needs an unstructured mesh (set it first)");
  size_t E = (size_t)c->mesh.nelem;
  if (!c->d_cet_sum) {
    if (cudaMalloc(&c->d_cet_sum, sizeof(double) * E) != cudaSuccess ||
        cudaMalloc(&c->d_cet_enc, sizeof(int) * E) != cudaSuccess) {
      cudaFree(c->d_cet_sum);
      c->d_cet_sum = nullptr;
      c->d_cet_enc = nullptr;
      return fail(c, FVC_ERR_OOM, "exposure-time accumulators");
    }
  }
  FVC_CUDA(c, cudaMemsetAsync(c->d_cet_sum, 0, sizeof(double) * E, c->stream));
  FVC_CUDA(c, cudaMemsetAsync(c->d_cet_enc, 0, sizeof(int) * E, c->stream));
  FVC_CUDA(c, cudaStreamSynchronize(c->stream));
  c->cet_sub = substeps;
  return FVC_OK;
}

extern "C" fvc_status fvc_cet_results(fvc_ctx* c, int ntracers, double* cet, double* met, int* enc) {
  if (!c) return FVC_ERR_ARG;
  if (!c->cet_sub) return fail(c, FVC_ERR_STATE, "exposure time is not enabled");
  fvc_status st;
  if ((st = use_device(c))) return st;
  size_t E = (size_t)c->mesh.nelem;
  if ((st = ensure_scratch(c, 16 * E))) return st;
  double* out = (double*)c->d_scratch;
  cet_results(c->mesh, cet_dev(c), ntracers, out, c->stream);
  if ((st = check_launch(c, "exposure-time results"))) return st;
  if (cet) FVC_CUDA(c, cudaMemcpyAsync(cet, out, 8 * E, cudaMemcpyDeviceToHost, c->stream));
  if (met) FVC_CUDA(c, cudaMemcpyAsync(met, out + E, 8 * E, cudaMemcpyDeviceToHost, c->stream));
  if (enc) FVC_CUDA(c, cudaMemcpyAsync(enc, c->d_cet_enc, 4 * E, cudaMemcpyDeviceToHost, c->stream));
  FVC_CUDA(c, cudaStreamSynchronize(c->stream));
  return FVC_OK;
}

extern "C" fvc_status fvc_tracer_residence(fvc_job* j, double launch_time, double stop_time, double* rt) {
  if (!j || j->kind != 1 || !rt) return FVC_ERR_ARG;
  fvc_ctx* c = j->ctx;
  fvc_status st;
  if ((st = use_device(c))) return st;
  if ((st = job_sync(j, "tracer advance"))) return st;
  size_t n = (size_t)j->t.n;
  if (n == 0) return FVC_OK;
  if ((st = ensure_scratch(c, 8 * n))) return st;
  double* d = (double*)c->d_scratch;
  tracer_residence(j->t, launch_time, stop_time, d, c->stream);
  if ((st = check_launch(c, "residence time"))) return st;
  j->stats.launches += 1;
  FVC_CUDA(c, cudaMemcpyAsync(rt, d, 8 * n, cudaMemcpyDeviceToHost, c->stream));
  FVC_CUDA(c, cudaStreamSynchronize(c->stream));
  return FVC_OK;
}

// ---------------------------------------------------------------- tracers

extern "C" fvc_status fvc_tracer_create(fvc_ctx* c, const fvc_tracer_spec* sp, int n, const double* seeds,
                                        fvc_job** out) {
  fvc_status st;
  if (!out || !sp) return fail(c, FVC_ERR_ARG, "null argument");
  *out = nullptr;
  if ((st = ready(c, false))) return st;
  if (n < 0 || (n > 0 && !seeds)) return fail(c, FVC_ERR_ARG, "bad seed array");
  fvc_job* j = new fvc_job();
  j->ctx = c;
  j->kind = 1;
  j->prec = c->prec;
  TracerDev& t = j->t;
  t.n = n;
  long nn = n > 0 ? n : 1;
  long nb = (nn + 1023) / 1024;
  int* left0 = nullptr;
  st = carve(c, &j->mem,
             {{(void**)&t.X, 24 * nn}, {(void**)&t.V, 24 * nn}, {(void**)&t.ldt, 8 * nn}, {(void**)&t.eid, 4 * nn},
              {(void**)&t.left, 4 * nn}, {(void**)&t.outX, 24 * nn},
              {(void**)&t.block_cnt, sizeof(int) * (2 * nb + 16) + sizeof(long long) * (nb / 1024 + 8)},
              {(void**)&t.live, 4 * nn}, {(void**)&j->live_alt, 4 * nn},
              {(void**)&left0, 4 * nn}},
             &j->mem_bytes);
  if (st) {
    delete j;
    return st;
  }
  cudaStream_t s = c->stream;
  if (n > 0) {
    job_events(j);
    cudaEventRecord(j->ev[3], s);
    FVC_CUDA(c, cudaMemcpyAsync(t.X, seeds, 24 * (size_t)n, cudaMemcpyHostToDevice, s));
    outside_domain_flags(c->mesh, n, t.X, left0, s);
    FVC_CUDA(c, cudaMemsetAsync(t.eid, 0xff, 4 * (size_t)n, s));
    if (c->mesh.mesh_type == 1) {
      int center = -1;
      if (sp->seed_chain == 1) {
        center = center_element(c, sp->center);
        if (center < -1) { fvc_job_destroy(j); return fail(c, FVC_ERR_CUDA, "centre search failed"); }
      }
      ChainArgs a{sp->seed_chain == 1 ? 2 : 1, n, {n, 1, 1}, sp->local_search_checking, center};
      if (sp->seed_chain == 1) j->stats.launches += 1;
      if ((st = run_chain(c, a, t.X, left0, t.eid, &j->stats.launches))) { fvc_job_destroy(j); return st; }
    }
    tracer_init_marks(c->mesh, t, left0, sp->seed_chain, s);
    j->stats.launches += 2;
    if ((st = check_launch(c, "tracer init"))) { fvc_job_destroy(j); return st; }
    if (j->prec) {
      pack_pairs(t.X, 3L * n, s);
      j->packed = true;
    }
    cudaEventRecord(j->ev[0], s);
    FVC_CUDA(c, cudaStreamSynchronize(s));
    j->stats.ms_setup += ev_ms(j->ev[3], j->ev[0]);  // seeds up, located, marked
  }
  *out = j;
  return FVC_OK;
}

extern "C" fvc_status fvc_tracer_launch(fvc_job* j, double t_start) {
  if (!j || j->kind != 1) return FVC_ERR_ARG;
  fvc_ctx* c = j->ctx;
  fvc_status st;
  if ((st = ready(c, true))) return st;
  if (j->prec != c->prec) return fail(c, FVC_ERR_STATE, "the job was created with another precision form");
  if ((st = mixed_ok(c))) return st;
  if ((st = cet_ok(c, j))) return st;
  if (c->cet_sub) {
    cet_release(j->t, cet_dev(c), c->stream);
    j->stats.launches += 1;
  }
  tracer_launch_vel(c->mesh, c->window, j->t, t_start, c->d_ctr, c->stream);
  if ((st = check_launch(c, "tracer launch"))) return st;
  j->stats.launches += 1;
  j->tlive_ready = false;  // the launch can mark tracers outside
  return finish(c, "tracer launch", nullptr);
}

// The job's own counters (FTLE intervals and tracer advances run on them
// asynchronously; job_sync reads and clears them).
static fvc_status job_counters(fvc_job* j) {
  if (j->d_ctr) return FVC_OK;
  fvc_ctx* c = j->ctx;
  if (cudaMalloc(&j->d_ctr, sizeof(DevCounters)) != cudaSuccess) return fail(c, FVC_ERR_OOM, "job counters");
  FVC_CUDA(c, cudaMemsetAsync(j->d_ctr, 0, sizeof(DevCounters), c->stream));
  return FVC_OK;
}

// Three events of an asynchronous call, accounted by job_sync as (main
// start, main end, early end).
static fvc_status job_event_triple(fvc_job* j, cudaEvent_t ev[3]) {
  for (int k = 0; k < 3; k++) {
    if (!j->spare.empty()) {
      ev[k] = j->spare.back();
      j->spare.pop_back();
    } else if (cudaEventCreate(&ev[k]) != cudaSuccess) {
      return fail(j->ctx, FVC_ERR_CUDA, "event creation failed");
    }
    j->pend.push_back(ev[k]);
  }
  return FVC_OK;
}

extern "C" fvc_status fvc_tracer_advance(fvc_job* j, double t1, double t2, long long* steps) {
  if (!j || j->kind != 1) return FVC_ERR_ARG;
  fvc_ctx* c = j->ctx;
  fvc_status st;
  if ((st = ready(c, true))) return st;
  job_events(j);
  if (j->prec != c->prec) return fail(c, FVC_ERR_STATE, "the job was created with another precision form");
  if ((st = mixed_ok(c))) return st;
  if ((st = cet_ok(c, j))) return st;
  if ((st = prepare_slots(c, t1, t2))) return st;
  if ((st = job_counters(j))) return st;
  cudaEvent_t ev[3];
  if ((st = job_event_triple(j, ev))) return st;
  // the live list: built by the previous advance, or compacted here (the
  // first advance, after a launch, or with exposure time, whose kernel does
  // not build it)
  const bool fused = !c->cet_sub && j->t.n > 0;
  const int a = j->tgen % 3;
  bool compacted = false;
  if (!fused || !j->tlive_ready || j->tlive_extrap != c->integ.extrapolate) {
    compact_live(j->t.n, j->t.ldt, j->t.left, c->integ.extrapolate, j->t.live, nullptr, j->t.block_cnt, j->d_ctr,
                 c->stream);
    compacted = true;
    if (fused) {
      FVC_CUDA(c, cudaMemcpyAsync(&j->d_ctr->lcnt[a], &j->d_ctr->nlive, sizeof(int), cudaMemcpyDeviceToDevice,
                                  c->stream));
      FVC_CUDA(c, cudaMemsetAsync(&j->d_ctr->lcur[a], 0, sizeof(int), c->stream));
      FVC_CUDA(c, cudaMemsetAsync(&j->d_ctr->lcnt[(a + 1) % 3], 0, sizeof(int), c->stream));
    }
  }
  TracerDev t = j->t;
  t.live_next = fused ? j->live_alt : nullptr;
  t.gen = j->tgen;
  cudaEventRecord(ev[0], c->stream);
  if (c->cet_sub) tracer_advance_cet(c->mesh, c->window, c->integ, t, t1, t2, cet_dev(c), j->d_ctr, c->stream);
  else tracer_advance(c->mesh, c->window, c->integ, t, t1, t2, j->d_ctr, c->stream);
  cudaEventRecord(ev[1], c->stream);
  if (fused) {
    std::swap(j->t.live, j->live_alt);
    j->tgen++;
    j->tlive_ready = true;
    j->tlive_extrap = c->integ.extrapolate;
  } else {
    j->tlive_ready = false;
  }
  cudaEventRecord(ev[2], c->stream);
  if ((st = check_launch(c, "tracer advance"))) return st;
  j->stats.intervals++;
  j->stats.launches += 1 + (compacted ? 4 : 0) + c->aux_launches;
  c->aux_launches = 0;
  if (!steps) return FVC_OK;  // asynchronous: accounted by the next call that waits
  const long long before = j->stats.steps_main;
  st = job_sync(j, "tracer advance");
  *steps = j->stats.steps_main - before;
  return st;
}

// ------------------------------------------------------ asynchronous outputs

// Frees the output ring (its device and page-locked blocks start at slot 0).
static void out_free(fvc_ctx* c) {
  if (c->out_stream) cudaStreamSynchronize(c->out_stream);
  cudaFree(c->out[0].d);
  cudaFreeHost(c->out[0].h);
  for (auto& o : c->out) {
    o.d = nullptr;
    o.h = nullptr;
    o.hc = nullptr;
    if (o.copied) cudaEventDestroy(o.copied);
    if (o.compacted) cudaEventDestroy(o.compacted);
    o.copied = o.compacted = nullptr;
    o.ticket = -1;
    o.busy = false;
  }
  c->out_rows_cap = 0;
  if (c->out_stream) cudaStreamDestroy(c->out_stream);
  c->out_stream = nullptr;
}

// The ring's buffers with room for `rows` rows a slot: one device block and
// one page-locked block (positions, then the slots' counts and statuses).
static fvc_status out_reserve(fvc_ctx* c, size_t rows) {
  if (rows <= c->out_rows_cap && c->out[0].d) return FVC_OK;
  {
    std::lock_guard<std::mutex> lock(c->out_mu);
    for (auto& o : c->out)
      if (o.busy) return fail(c, FVC_ERR_STATE, "tracer outputs of a smaller job are still held: release them first");
  }
  if (!c->out_stream && cudaStreamCreateWithFlags(&c->out_stream, cudaStreamNonBlocking) != cudaSuccess)
    return fail(c, FVC_ERR_CUDA, "output stream");
  cudaStreamSynchronize(c->out_stream);
  void* hold = c->out[0].h;
  cudaFree(c->out[0].d);
  cudaFreeHost(hold);
  for (auto& o : c->out) {
    o.d = nullptr;
    o.h = nullptr;
    o.hc = nullptr;
  }
  const size_t slot = al256(24 * rows);
  const int ns = FVC_TRACER_OUTPUT_SLOTS;
  unsigned char *d = nullptr, *h = nullptr;
  if (cudaMalloc(&d, slot * ns) != cudaSuccess) return fail(c, FVC_ERR_OOM, "tracer output ring (device)");
  if (cudaMallocHost(&h, slot * ns + 256) != cudaSuccess) {
    cudaFree(d);
    return fail(c, FVC_ERR_OOM, "tracer output ring (page-locked host)");
  }
  for (int k = 0; k < ns; k++) {
    auto& o = c->out[k];
    o.d = (double*)(d + k * slot);
    o.h = (double*)(h + k * slot);
    o.hc = (int*)(h + ns * slot) + 2 * k;
    o.ticket = -1;
    o.busy = false;
    if ((!o.copied && cudaEventCreateWithFlags(&o.copied, cudaEventDisableTiming) != cudaSuccess) ||
        (!o.compacted && cudaEventCreateWithFlags(&o.compacted, cudaEventDisableTiming) != cudaSuccess))
      return fail(c, FVC_ERR_CUDA, "output event");
  }
  c->out_rows_cap = rows;
  return FVC_OK;
}

extern "C" fvc_status fvc_tracer_output_begin(fvc_job* j, int always, long long* ticket) {
  if (!j || j->kind != 1 || !ticket) return FVC_ERR_ARG;
  fvc_ctx* c = j->ctx;
  fvc_status st;
  if ((st = use_device(c))) return st;
  if ((st = job_counters(j))) return st;
  const size_t n = (size_t)j->t.n;
  if ((st = out_reserve(c, n > 0 ? n : 1))) return st;
  int k;
  {
    std::lock_guard<std::mutex> lock(c->out_mu);
    k = (int)(c->out_next % FVC_TRACER_OUTPUT_SLOTS);
    if (c->out[k].busy)
      return fail(c, FVC_ERR_STATE, "all %d tracer output slots are held: release output %lld first",
                  FVC_TRACER_OUTPUT_SLOTS, c->out[k].ticket);
    // completed outputs of this job bound the next one's count
    for (auto& o : c->out)
      if (o.n == (long long)n && o.ticket >= 0 && o.hc && cudaEventQuery(o.copied) == cudaSuccess &&
          o.tag == (const void*)j && (j->out_bound < 0 || o.hc[0] < j->out_bound))
        j->out_bound = o.hc[0];
    cudaGetLastError();  // cudaEventQuery's cudaErrorNotReady is not an error
  }
  auto& o = c->out[k];
  cudaStream_t s = c->stream;
  // the slot's previous copy must be done before its buffer is rewritten
  FVC_CUDA(c, cudaStreamWaitEvent(s, o.copied, 0));
  TracerDev t = j->t;
  t.outX = o.d;
  const int nl = tracer_compact(t, always, j->d_ctr, s, j->packed);
  if ((st = check_launch(c, "tracer output"))) return st;
  j->stats.launches += nl;
  FVC_CUDA(c, cudaMemcpyAsync(o.hc, &j->d_ctr->count, sizeof(int), cudaMemcpyDeviceToHost, s));
  FVC_CUDA(c, cudaMemcpyAsync(o.hc + 1, &j->d_ctr->status, sizeof(int), cudaMemcpyDeviceToHost, s));
  // the copy runs on the side stream after the compaction; its length is a
  // bound on the count (the last completed output's count, else every
  // tracer), and wait() copies the rest in the rare case the bound was short
  const long long rows = j->out_bound >= 0 ? j->out_bound : (long long)n;
  FVC_CUDA(c, cudaEventRecord(o.compacted, s));
  FVC_CUDA(c, cudaStreamWaitEvent(c->out_stream, o.compacted, 0));
  if (rows > 0)
    FVC_CUDA(c, cudaMemcpyAsync(o.h, o.d, 24 * (size_t)rows, cudaMemcpyDeviceToHost, c->out_stream));
  FVC_CUDA(c, cudaEventRecord(o.copied, c->out_stream));
  {
    std::lock_guard<std::mutex> lock(c->out_mu);
    o.rows = rows;
    o.n = (long long)n;
    o.tag = (const void*)j;
    o.ticket = c->out_next++;
    o.busy = true;
    *ticket = o.ticket;
  }
  return FVC_OK;
}

static fvc_ctx::OutSlot* out_find(fvc_ctx* c, long long ticket) {
  for (auto& o : c->out)
    if (o.busy && o.ticket == ticket) return &o;
  return nullptr;
}

extern "C" fvc_status fvc_tracer_output_wait(fvc_ctx* c, long long ticket, const double** X, long long* count) {
  if (!c || !X || !count) return FVC_ERR_ARG;
  fvc_ctx::OutSlot* o;
  {
    std::lock_guard<std::mutex> lock(c->out_mu);
    o = out_find(c, ticket);
  }
  if (!o) return FVC_ERR_STATE;
  if (cudaSetDevice(c->device) != cudaSuccess || cudaEventSynchronize(o->copied) != cudaSuccess)
    return FVC_ERR_CUDA;
  const int status = o->hc[1];
  if (status & PT_ERR_STATE) return FVC_ERR_STATE;
  if (status & PT_ERR_TLOC) return FVC_ERR_TLOC;
  if (status & (PT_ERR_WALK | PT_ERR_CET)) return FVC_ERR_WALK;
  const long long cnt = o->hc[0];
  if (cnt > o->rows) {
    // the bound was short: the rest of the rows, from the slot (intact
    // until released), on a stream of this call's own
    cudaStream_t s2 = nullptr;
    if (cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking) != cudaSuccess) return FVC_ERR_CUDA;
    cudaError_t e = cudaMemcpyAsync(o->h + 3 * o->rows, o->d + 3 * o->rows, 24 * (size_t)(cnt - o->rows),
                                    cudaMemcpyDeviceToHost, s2);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s2);
    cudaStreamDestroy(s2);
    if (e != cudaSuccess) return FVC_ERR_CUDA;
    std::lock_guard<std::mutex> lock(c->out_mu);
    o->rows = cnt;
  }
  *X = o->h;
  *count = cnt;
  return FVC_OK;
}

extern "C" fvc_status fvc_tracer_output_release(fvc_ctx* c, long long ticket) {
  if (!c) return FVC_ERR_ARG;
  std::lock_guard<std::mutex> lock(c->out_mu);
  fvc_ctx::OutSlot* o = out_find(c, ticket);
  if (!o) return FVC_ERR_STATE;
  o->busy = false;
  return FVC_OK;
}

extern "C" fvc_status fvc_tracer_snapshot(fvc_job* j, int always, double* X_out, long long* count) {
  if (!j || j->kind != 1 || !count) return FVC_ERR_ARG;
  fvc_ctx* c = j->ctx;
  fvc_status st;
  if ((st = use_device(c))) return st;
  if ((st = job_sync(j, "tracer advance"))) return st;  // faults of queued advances
  j->stats.launches += tracer_compact(j->t, always, c->d_ctr, c->stream);
  if ((st = check_launch(c, "tracer snapshot"))) return st;
  int cnt = 0;
  FVC_CUDA(c, cudaMemcpyAsync(&cnt, &c->d_ctr->count, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  FVC_CUDA(c, cudaStreamSynchronize(c->stream));
  *count = cnt;
  if (X_out && cnt > 0)
    FVC_CUDA(c, cudaMemcpyAsync(X_out, j->t.outX, 24 * (size_t)cnt, cudaMemcpyDeviceToHost, c->stream));
  FVC_CUDA(c, cudaStreamSynchronize(c->stream));
  if (X_out && j->packed) unpack_host(X_out, 3 * (size_t)cnt);
  return FVC_OK;
}

extern "C" fvc_status fvc_tracer_get_state(fvc_job* j, double* X, int* eid, int* left, double* ldt) {
  if (!j || j->kind != 1) return FVC_ERR_ARG;
  fvc_ctx* c = j->ctx;
  fvc_status st;
  if ((st = use_device(c))) return st;
  if ((st = job_sync(j, "tracer advance"))) return st;
  size_t n = (size_t)j->t.n;
  cudaStream_t s = c->stream;
  if (n == 0) return FVC_OK;
  if (X) FVC_CUDA(c, cudaMemcpyAsync(X, j->t.X, 24 * n, cudaMemcpyDeviceToHost, s));
  if (eid) FVC_CUDA(c, cudaMemcpyAsync(eid, j->t.eid, 4 * n, cudaMemcpyDeviceToHost, s));
  if (left) FVC_CUDA(c, cudaMemcpyAsync(left, j->t.left, 4 * n, cudaMemcpyDeviceToHost, s));
  if (ldt) FVC_CUDA(c, cudaMemcpyAsync(ldt, j->t.ldt, 8 * n, cudaMemcpyDeviceToHost, s));
  FVC_CUDA(c, cudaStreamSynchronize(s));
  if (X && j->packed) unpack_host(X, 3 * n);
  return FVC_OK;
}

// ------------------------------------------------- allocation-free advection
//
// fvc_advect_noalloc serves callers that may not allocate device memory while
// they run (an application whose own pool allocator owns the rest of the GPU,
// or a code path where the device synchronisation of a cudaMalloc is not
// allowed).  Its scratch is this one file-scope array, which every GPU that
// loads the library holds until the process exits.  Layout, each part
// 256-byte aligned: the step counters, then X, V, eid, left and ldt sized for
// FVC_NOALLOC_MAX_POINTS, then the stage-time velocity table in the rest.
// Every call on a device shares the array and finds the previous call's bytes
// in it: the counters are cleared at the start of each call, and every other
// byte a call reads it has written before.

static __device__ __align__(256) unsigned char g_noalloc_scratch[FVC_NOALLOC_SCRATCH_BYTES];

static constexpr size_t na_al(size_t b) { return (b + 255) & ~(size_t)255; }
static constexpr size_t NA_MAXN = FVC_NOALLOC_MAX_POINTS;
static constexpr size_t NA_CTR = na_al(sizeof(DevCounters));
static constexpr size_t NA_X = na_al(sizeof(double) * 3 * NA_MAXN), NA_I = na_al(sizeof(int) * NA_MAXN),
                        NA_D = na_al(sizeof(double) * NA_MAXN);
static constexpr size_t NA_VT = NA_CTR + 2 * NA_X + 2 * NA_I + NA_D;  // start of the velocity table
static_assert(NA_VT < (size_t)FVC_NOALLOC_SCRATCH_BYTES, "no room left for the stage-time table");

#define FVC_NOALLOC_MAX_DEVICES 64
static std::mutex g_noalloc_mu;
static unsigned char* g_noalloc_base[FVC_NOALLOC_MAX_DEVICES];

// The array's device address on the context's device (current when this is
// called).  In host code g_noalloc_scratch only names the array; the address
// the kernels get is the one cudaGetSymbolAddress returns, looked up on a
// device's first call and kept for the process's life (a cudaDeviceReset
// would make it stale; the header tells callers not to reset).
static fvc_status noalloc_base(fvc_ctx* c, unsigned char** base) {
  if (c->device >= FVC_NOALLOC_MAX_DEVICES)
    return fail(c, FVC_ERR_ARG, "fvc_advect_noalloc supports devices 0..%d", FVC_NOALLOC_MAX_DEVICES - 1);
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  unsigned char*& b = g_noalloc_base[c->device];
  if (!b) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return fail(c, FVC_ERR_CUDA, "device address of the fvc_advect_noalloc scratch: %s", cudaGetErrorString(e));
    b = (unsigned char*)p;
  }
  *base = b;
  return FVC_OK;
}

// The stage-time slots of prepare_slots, computed the same way, with the
// table limited to the slots that fit in vt_bytes.  Slots are hints that the
// kernels check against the time they compute, so a shorter table gives the
// same results.
static void noalloc_slots(const fvc_ctx* c, DevWindow& w, double t1, double t2, double4_32a* vt,
                          size_t vt_bytes) {
  int cap = FVC_MAX_SLOTS;
  if (c->mesh.mesh_type == 1) {
    size_t per = sizeof(double4_32a) * (size_t)c->mesh.nnodes;
    size_t fit = per ? vt_bytes / per : 0;
    if (fit < (size_t)cap) cap = (int)fit;
  }
  int n = 0;
  auto add = [&](double tq) {
    if (n >= cap) return false;
    double tloc = (tq - w.tmin) / (w.tmax - w.tmin);
    if ((tloc > 1 + 1.0e-10) || (tloc < 0 - 1.0e-10)) return false;
    w.tq[n] = tq;
    w.tl[n] = tloc;
    n++;
    return true;
  };
  double tc = t1, h = (t2 - t1) >= 0.0 ? fabs(c->integ.h) : -fabs(c->integ.h);
  bool ok = true;
  while ((tc - t2) * (t2 - t1) < 0.0) {
    if ((tc + h - t2) * (tc + h - t1) > 0.0) h = (t2 - t1) >= 0.0 ? fabs(t2 - tc) : -fabs(t2 - tc);
    if (!add(tc) || !add(tc + h / 2)) {
      ok = false;
      break;
    }
    tc = tc + h;
  }
  if (ok) add(tc);
  w.nslots = n;
  w.vt = vt;
  w.vt_stride = c->mesh.nnodes;
}

extern "C" fvc_status fvc_advect_noalloc(fvc_ctx* c, int n, double* X, double* V, int* eid, int* left,
                                         double* ldt, double t0, double t1, long long* steps) {
  fvc_status st;
  if ((st = ready(c, true))) return st;
  if (n < 0 || (n > 0 && (!X || !left || !ldt))) return fail(c, FVC_ERR_ARG, "bad arrays");
  if (n > FVC_NOALLOC_MAX_POINTS)
    return fail(c, FVC_ERR_ARG,
                "fvc_advect_noalloc: %d points exceed its fixed scratch (at most %d points a call); "
                "split the call or use fvc_advect", n, FVC_NOALLOC_MAX_POINTS);
  if (c->mesh.mesh_type == 1 && n > 0 && !eid) return fail(c, FVC_ERR_ARG, "unstructured advection needs element ids");
  if (c->integ.extrapolate && n > 0 && !V) return fail(c, FVC_ERR_ARG, "extrapolation needs V");
  if (c->prec) return fail(c, FVC_ERR_ARG, "fvc_advect_noalloc runs the FP64 form only");
  if ((st = mixed_ok(c))) return st;
  if (steps) *steps = 0;
  if (n == 0) return FVC_OK;
  unsigned char* base = nullptr;
  if ((st = noalloc_base(c, &base))) return st;
  DevCounters* ctr = (DevCounters*)base;
  double* dX = (double*)(base + NA_CTR);
  double* dV = (double*)(base + NA_CTR + NA_X);
  int* de = (int*)(base + NA_CTR + 2 * NA_X);
  int* dl = (int*)(base + NA_CTR + 2 * NA_X + NA_I);
  double* dt = (double*)(base + NA_CTR + 2 * NA_X + 2 * NA_I);
  double4_32a* vt = (double4_32a*)(base + NA_VT);
  cudaStream_t s = c->stream;
  FVC_CUDA(c, cudaMemsetAsync(ctr, 0, sizeof(DevCounters), s));
  FVC_CUDA(c, cudaMemcpyAsync(dX, X, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s));
  if (V) FVC_CUDA(c, cudaMemcpyAsync(dV, V, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s));
  if (eid) FVC_CUDA(c, cudaMemcpyAsync(de, eid, sizeof(int) * n, cudaMemcpyHostToDevice, s));
  FVC_CUDA(c, cudaMemcpyAsync(dl, left, sizeof(int) * n, cudaMemcpyHostToDevice, s));
  FVC_CUDA(c, cudaMemcpyAsync(dt, ldt, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  DevWindow w = c->window;  // the context's window is left as it is
  noalloc_slots(c, w, t0, t1, vt, (size_t)FVC_NOALLOC_SCRATCH_BYTES - NA_VT);
  if (c->mesh.mesh_type == 1 && w.nslots > 0) {
    time_fields(c->mesh, w, vt, s);
    if ((st = check_launch(c, "time fields"))) return st;
  }
  launch_advect(c->mesh, w, c->integ, n, dX, V ? dV : nullptr, eid ? de : nullptr, dl, dt, t0, t1, ctr, s);
  if ((st = check_launch(c, "advect"))) return st;
  FVC_CUDA(c, cudaMemcpyAsync(X, dX, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, s));
  if (V) FVC_CUDA(c, cudaMemcpyAsync(V, dV, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, s));
  if (eid) FVC_CUDA(c, cudaMemcpyAsync(eid, de, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
  FVC_CUDA(c, cudaMemcpyAsync(left, dl, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
  FVC_CUDA(c, cudaMemcpyAsync(ldt, dt, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  DevCounters h{};
  FVC_CUDA(c, cudaMemcpyAsync(&h, ctr, sizeof(h), cudaMemcpyDeviceToHost, s));
  FVC_CUDA(c, cudaStreamSynchronize(s));
  if (steps) *steps = (long long)(h.steps + h.steps_early);
  if (h.status & PT_ERR_STATE)
    return fail(c, FVC_ERR_STATE, "advect: a point that had left the domain was advected");
  if (h.status & PT_ERR_TLOC) return fail(c, FVC_ERR_TLOC, "advect: query time outside the loaded frame interval");
  if (h.status & PT_ERR_WALK)
    return fail(c, FVC_ERR_WALK, "advect: neighbour walk failed (indeterminate neighbour or hop cap)");
  return FVC_OK;
}
