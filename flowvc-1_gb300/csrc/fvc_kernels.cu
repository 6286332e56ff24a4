// fvc_kernels.cu -- sm_103a kernels of the flowVC advection engine: mesh
// preprocessing, bucket grid, seed-location chain, FTLE bookkeeping and the
// tracer output compaction; the integrator kernels live in fvc_variant_*.cu.
//
// Built with --fmad=false: the FP64 paths must round every multiply and add
// separately to reproduce ompVC's results bit for bit (see fvc_device.cuh).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>
#include <vector>

#include "fvc_device.cuh"
#include "fvc_advect_impl.cuh"
#include "fvc_mixed_impl.cuh"
#include "fvc_ftle_math.cuh"
#include "fvc_kernels.h"

namespace fvc {


static inline unsigned nblk(long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

// ============================================================ mesh geometry

// Natural-coordinate map of every element, from the expressions of
// ompVC/velocity.c:497-510 (3D) and 529-535 (2D), with the element's node ids
// in the same record so one gather serves the containment test and the
// interpolation (layout in fvc_device.cuh, struct Geo).
template <int DIMS>
__global__ void k_geometry(DevMesh m, double* geom, float* geo32, float4* geo32lo) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m.nelem) return;
  int4 nd = m.elem[2 * (long)e];
  double4_32a p0 = m.nodes[nd.x], p1 = m.nodes[nd.y], p2 = m.nodes[nd.z];
  double x0 = p0.x, y0 = p0.y, x1 = p1.x, y1 = p1.y, x2 = p2.x, y2 = p2.y;
  if (DIMS == 3) {
    double4_32a p3 = m.nodes[nd.w];
    double z0 = p0.z, z1 = p1.z, z2 = p2.z, x3 = p3.x, y3 = p3.y, z3 = p3.z;
    double* g = geom + (long)e * 16;
    g[0] = (z3 - z0) * (y2 - y3) - (z2 - z3) * (y3 - y0);   // a11
    g[3] = (z3 - z0) * (y0 - y1) - (z0 - z1) * (y3 - y0);   // a21
    g[6] = (z1 - z2) * (y0 - y1) - (z0 - z1) * (y1 - y2);   // a31
    g[1] = (x3 - x0) * (z2 - z3) - (x2 - x3) * (z3 - z0);   // a12
    g[4] = (x3 - x0) * (z0 - z1) - (x0 - x1) * (z3 - z0);   // a22
    g[7] = (x1 - x2) * (z0 - z1) - (x0 - x1) * (z1 - z2);   // a32
    g[2] = (y3 - y0) * (x2 - x3) - (y2 - y3) * (x3 - x0);   // a13
    g[5] = (y3 - y0) * (x0 - x1) - (y0 - y1) * (x3 - x0);   // a23
    g[8] = (y1 - y2) * (x0 - x1) - (y0 - y1) * (x1 - x2);   // a33
    g[9] = (x1 - x0) * ((y2 - y0) * (z3 - z0) - (z2 - z0) * (y3 - y0)) +
           (x2 - x0) * ((y0 - y1) * (z3 - z0) - (z0 - z1) * (y3 - y0)) +
           (x3 - x0) * ((y1 - y0) * (z2 - z0) - (z1 - z0) * (y2 - y0));  // V
    g[10] = x0;
    g[11] = y0;
    g[12] = z0;
    g[13] = rcp_for_div(g[9]);
    reinterpret_cast<int4*>(g + 14)[0] = nd;
    // FP32 copy for the walk's pre-check: a11..a33, 1/V, x0 y0 z0, and the
    // scale A = sum |a_ij| / |V| of the coordinates' error per unit offset error
    float* q = geo32 + (long)e * 16;
    for (int c = 0; c < 9; c++) q[c] = (float)g[c];
    q[9] = (float)(1.0 / g[9]);
    q[10] = (float)x0;
    q[11] = (float)y0;
    q[12] = (float)z0;
    double sa = 0.0;
    for (int c = 0; c < 9; c++) sa += fabs(g[c]);
    q[13] = (float)(sa / fabs(g[9]) * (1.0 + 1e-6));
    q[14] = q[15] = 0.f;
    geo32lo[e] = make_float4((float)(x0 - (double)q[10]), (float)(y0 - (double)q[11]), (float)(z0 - (double)q[12]), 0.f);
  } else {
    double* g = geom + (long)e * 12;
    g[0] = y2 - y0;  // a11
    g[1] = x0 - x2;  // a12
    g[2] = y0 - y1;  // a21
    g[3] = x1 - x0;  // a22
    g[4] = (x1 - x0) * (y2 - y0) - (x2 - x0) * (y1 - y0);  // V
    g[5] = x0;
    g[6] = y0;
    g[7] = rcp_for_div(g[4]);
    reinterpret_cast<int4*>(g + 8)[0] = nd;
    g[10] = g[11] = 0.0;
    float* q = geo32 + (long)e * 16;
    for (int c = 0; c < 4; c++) q[c] = (float)g[c];
    q[4] = (float)(1.0 / g[4]);
    q[5] = (float)x0;
    q[6] = (float)y0;
    double sa = fabs(g[0]) + fabs(g[1]) + fabs(g[2]) + fabs(g[3]);
    q[7] = (float)(sa / fabs(g[4]) * (1.0 + 1e-6));
    for (int c = 8; c < 16; c++) q[c] = 0.f;
    geo32lo[e] = make_float4((float)(x0 - (double)q[5]), (float)(y0 - (double)q[6]), 0.f, 0.f);
  }
}

// Element e's node ids and neighbours as given (4 + 4 ints) interleaved into
// the walk's layout (elem[2e] nodes, elem[2e + 1] neighbours; triangles
// repeat their third node and have no fourth neighbour), with the ranges
// checked: the lowest element with an id out of range goes to *bad.
__global__ void k_pack_elements(const int4* conn, const int4* adj, int nelem, int nnodes, int nv, int4* elem,
                                int* bad) {
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nelem) return;
  const int4 n = conn[e], a = adj[e];
  const bool ok = n.x >= 0 && n.x < nnodes && n.y >= 0 && n.y < nnodes && n.z >= 0 && n.z < nnodes &&
                  (nv < 4 || (n.w >= 0 && n.w < nnodes)) && a.x >= -1 && a.x < nelem && a.y >= -1 &&
                  a.y < nelem && a.z >= -1 && a.z < nelem && (nv < 4 || (a.w >= -1 && a.w < nelem));
  if (!ok) atomicMin(bad, (int)e);
  elem[2 * e] = make_int4(n.x, n.y, n.z, nv == 4 ? n.w : n.z);
  elem[2 * e + 1] = make_int4(a.x, a.y, a.z, nv == 4 ? a.w : -1);
}

void pack_elements(const int4* conn, const int4* adj, int nelem, int nnodes, int nv, int4* elem, int* bad,
                   cudaStream_t s) {
  k_pack_elements<<<nblk(nelem, 256), 256, 0, s>>>(conn, adj, nelem, nnodes, nv, elem, bad);
}

void launch_geometry(const DevMesh& m, double* geom, float* geo32, cudaStream_t s) {
  float4* lo = reinterpret_cast<float4*>(geo32 + 16L * m.nelem);
  if (m.dims == 3) k_geometry<3><<<nblk(m.nelem, 256), 256, 0, s>>>(m, geom, geo32, lo);
  else k_geometry<2><<<nblk(m.nelem, 256), 256, 0, s>>>(m, geom, geo32, lo);
}

// =============================================================== scans

// Exclusive prefix sum of a block's values (blockDim.x a multiple of 32,
// at most 1024); returns the block total in *total.
__device__ __forceinline__ long long block_exclusive_sum(long long v, long long* total) {
  __shared__ long long warp_sums[32];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  long long x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[wid] = x;
  __syncthreads();
  if (wid == 0) {
    long long ws = lane < nw ? warp_sums[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      long long y = __shfl_up_sync(0xffffffffu, ws, o);
      if (lane >= o) ws += y;
    }
    if (lane < nw) warp_sums[lane] = ws;
  }
  __syncthreads();
  long long off = wid > 0 ? warp_sums[wid - 1] : 0;
  *total = warp_sums[nw - 1];
  __syncthreads();
  return off + x - v;
}

// Block-wise exclusive scan of int counts into int offsets (two levels).
__global__ void k_scan_blocks(const int* in, int* out, int n, long long* block_tot) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  long long v = i < n ? in[i] : 0, tot;
  long long ex = block_exclusive_sum(v, &tot);
  if (i < n) out[i] = (int)ex;
  if (threadIdx.x == 0) block_tot[blockIdx.x] = tot;
}
__global__ void k_scan_tops(long long* block_tot, int nb, int* grand) {
  // single thread: nb is small (n / 1024)
  if (threadIdx.x || blockIdx.x) return;
  long long run = 0;
  for (int b = 0; b < nb; b++) {
    long long t = block_tot[b];
    block_tot[b] = run;
    run += t;
  }
  *grand = (int)run;
}
__global__ void k_scan_add(int* out, int n, const long long* block_off) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += (int)block_off[blockIdx.x];
}
// out[0..n-1] = exclusive scan of in, out[n] = total.  tmp holds n/1024+1 longs.
static void exclusive_scan(const int* in, int* out, int n, long long* tmp, cudaStream_t s) {
  unsigned nb = nblk(n, 1024);
  k_scan_blocks<<<nb, 1024, 0, s>>>(in, out, n, tmp);
  k_scan_tops<<<1, 32, 0, s>>>(tmp, (int)nb, out + n);
  k_scan_add<<<nb, 1024, 0, s>>>(out, n, tmp);
}

// ========================================================== bucket grid

template <int DIMS>
__device__ __forceinline__ void elem_cells(const DevMesh& m, const BucketGrid& g, int e, int lo[3],
                                           int hi[3]) {
  int4 nd = m.elem[2 * (long)e];
  double4_32a p[4];
  p[0] = m.nodes[nd.x];
  p[1] = m.nodes[nd.y];
  p[2] = m.nodes[nd.z];
  p[3] = DIMS == 3 ? m.nodes[nd.w] : p[2];
  double bmin[3] = {p[0].x, p[0].y, p[0].z}, bmax[3] = {p[0].x, p[0].y, p[0].z};
  for (int c = 1; c < 4; c++) {
    bmin[0] = fmin(bmin[0], p[c].x); bmax[0] = fmax(bmax[0], p[c].x);
    bmin[1] = fmin(bmin[1], p[c].y); bmax[1] = fmax(bmax[1], p[c].y);
    bmin[2] = fmin(bmin[2], p[c].z); bmax[2] = fmax(bmax[2], p[c].z);
  }
  // A point passes the containment test d > -TINY only within ~1e-10 of the
  // element (in units of its size); pad the box by 1e-7 of its extent.
  double ext = fmax(bmax[0] - bmin[0], fmax(bmax[1] - bmin[1], DIMS == 3 ? bmax[2] - bmin[2] : 0.0));
  double pad = 1e-7 * ext + 1e-300;
  for (int a = 0; a < 3; a++) {
    if (a == 2 && DIMS == 2) { lo[a] = hi[a] = 0; continue; }
    int l = (int)floor((bmin[a] - pad - g.lo[a]) * g.inv[a]);
    int h = (int)floor((bmax[a] + pad - g.lo[a]) * g.inv[a]);
    lo[a] = max(0, min(g.n[a] - 1, l));
    hi[a] = max(0, min(g.n[a] - 1, h));
  }
}

template <int DIMS>
__global__ void k_bucket_count(DevMesh m, BucketGrid g, int* cnt) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m.nelem) return;
  int lo[3], hi[3];
  elem_cells<DIMS>(m, g, e, lo, hi);
  for (int k = lo[2]; k <= hi[2]; k++)
    for (int j = lo[1]; j <= hi[1]; j++)
      for (int i = lo[0]; i <= hi[0]; i++) atomicAdd(&cnt[((long)k * g.n[1] + j) * g.n[0] + i], 1);
}

template <int DIMS>
__global__ void k_bucket_fill(DevMesh m, BucketGrid g, const int* start, int* cursor, int* ids) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m.nelem) return;
  int lo[3], hi[3];
  elem_cells<DIMS>(m, g, e, lo, hi);
  for (int k = lo[2]; k <= hi[2]; k++)
    for (int j = lo[1]; j <= hi[1]; j++)
      for (int i = lo[0]; i <= hi[0]; i++) {
        long c = ((long)k * g.n[1] + j) * g.n[0] + i;
        ids[start[c] + atomicAdd(&cursor[c], 1)] = e;
      }
}

// ascending element ids within each cell, so the first hit is the lowest id
__global__ void k_bucket_sort(const int* start, int* ids, int ncells) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  int b = start[c], e = start[c + 1];
  for (int i = b + 1; i < e; i++) {
    int v = ids[i], j = i - 1;
    while (j >= b && ids[j] > v) {
      ids[j + 1] = ids[j];
      j--;
    }
    ids[j + 1] = v;
  }
}

long long bucket_count(const DevMesh& m, BucketGrid& g, int* cell_count, int ncells, int* d_total,
                       cudaStream_t s) {
  (void)d_total;
  cudaMemsetAsync(cell_count, 0, sizeof(int) * (size_t)ncells, s);
  if (m.dims == 3) k_bucket_count<3><<<nblk(m.nelem, 256), 256, 0, s>>>(m, g, cell_count);
  else k_bucket_count<2><<<nblk(m.nelem, 256), 256, 0, s>>>(m, g, cell_count);
  return 0;
}

void bucket_fill(const DevMesh& m, const BucketGrid& g, int* cell_start, int* cursor, int* ids,
                 int ncells, int* scan_tmp, cudaStream_t s) {
  (void)scan_tmp;
  cudaMemsetAsync(cursor, 0, sizeof(int) * (size_t)ncells, s);
  if (m.dims == 3) k_bucket_fill<3><<<nblk(m.nelem, 256), 256, 0, s>>>(m, g, cell_start, cursor, ids);
  else k_bucket_fill<2><<<nblk(m.nelem, 256), 256, 0, s>>>(m, g, cell_start, cursor, ids);
  k_bucket_sort<<<nblk(ncells, 256), 256, 0, s>>>(cell_start, ids, ncells);
}

// exported scan for the API layer (cell offsets)
void scan_counts(const int* in, int* out, int n, long long* tmp, cudaStream_t s) {
  exclusive_scan(in, out, n, tmp, s);
}

template <int DIMS>
__global__ void k_global(DevMesh m, BucketGrid g, int n, const double* X, const int* skip, int* out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (skip && skip[i]) {
    out[i] = -1;
    return;
  }
  double x[3] = {X[3 * (long)i], X[3 * (long)i + 1], X[3 * (long)i + 2]};
  out[i] = global_find<DIMS>(m, g, x);
}

// The global search's answer and whether it is the only element that
// passes the containment test d > -TINY at the point.  Every element that can
// pass it is a candidate of the point's bucket (their padded boxes hold the
// point), so scanning the whole list decides it.  When it is the only one, a
// neighbour walk from any start can stop nowhere else: it ends there, or
// leaves the mesh (and with LocalSearchChecking the global search answers).
template <int DIMS>
__global__ void k_global_unique(DevMesh m, BucketGrid g, int n, const double* X, const int* skip, int* out,
                                int* unique) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int first = -1, hits = 0;
  if (!(skip && skip[i])) {
    const double x[3] = {X[3 * (long)i], X[3 * (long)i + 1], X[3 * (long)i + 2]};
    int c[3];
    bool in = true;
    for (int a = 0; a < 3; a++) {
      if (a == 2 && DIMS == 2) { c[a] = 0; continue; }
      double f = (x[a] - g.lo[a]) * g.inv[a];
      if (!(f >= 0.0) || f >= (double)g.n[a]) { in = false; break; }
      c[a] = min(g.n[a] - 1, (int)f);
    }
    if (in) {
      const long cell = ((long)c[2] * g.n[1] + c[1]) * g.n[0] + c[0];
      const int b = __ldg(g.start + cell), e = __ldg(g.start + cell + 1);
      const PosF P = pos_f32(x);
      for (int k = b; k < e && hits < 2; k++) {
        const int el = __ldg(g.ids + k);
        const int qs = quick_hop<DIMS>(m, el, P);
        if (qs >= 0) continue;
        if (qs == -2 || contains<DIMS>(m, el, x)) {
          if (!hits) first = el;
          hits++;
        }
      }
    }
  }
  out[i] = first;
  unique[i] = hits == 1;
}

void launch_global_search(const DevMesh& m, const BucketGrid& g, int n, const double* X,
                          const int* skip, int* out, cudaStream_t s) {
  if (n <= 0) return;
  if (m.dims == 3) k_global<3><<<nblk(n, 128), 128, 0, s>>>(m, g, n, X, skip, out);
  else k_global<2><<<nblk(n, 128), 128, 0, s>>>(m, g, n, X, skip, out);
}

// ============================================================ step level

template <int D>
__global__ void k_local(DevMesh m, int n, const double* X, const int* guess, int* out, DevCounters* ctr) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  int err = 0;
  if (i < n) {
    double x[3] = {X[3 * i], X[3 * i + 1], X[3 * i + 2]};
    out[i] = locate_once<D>(m, x, guess[i], err);
  }
  flush_counters(&ctr->steps, &ctr->status, 0, err);
}

void launch_local_search(const DevMesh& m, int n, const double* X, const int* guess, int* out,
                         DevCounters* ctr, cudaStream_t s) {
  if (n <= 0) return;
  if (m.dims == 3) k_local<3><<<nblk(n, 128), 128, 0, s>>>(m, n, X, guess, out, ctr);
  else k_local<2><<<nblk(n, 128), 128, 0, s>>>(m, n, X, guess, out, ctr);
}

__global__ void k_outside(DevMesh m, int n, const double* X, int* left0) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double x[3] = {X[3 * i], X[3 * i + 1], X[3 * i + 2]};
  left0[i] = outside_domain(m, x);
}

void outside_domain_flags(const DevMesh& m, int n, const double* X, int* left0, cudaStream_t s) {
  if (n <= 0) return;
  k_outside<<<nblk(n, 256), 256, 0, s>>>(m, n, X, left0);
}

// (1 - tloc) * U0 + tloc * U1 at every node for every stage time of the call
// (the expression of ompVC/velocity.c:547-571), so stage evaluations read it.
// One thread per node: both frames' values are read once and every slot's
// field written from them.
__global__ void k_time_fields(DevWindow w, long nnodes, double4_32a* vt) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nnodes) return;
  const double4_32a a = w.f0[i], b = w.f1[i];
  for (int sl = 0; sl < w.nslots; sl++) {
    const double tloc = w.tl[sl];
    vt[(long)sl * nnodes + i] = make_double4_32a((1 - tloc) * a.x + tloc * b.x, (1 - tloc) * a.y + tloc * b.y,
                                                 (1 - tloc) * a.z + tloc * b.z, 0.0);
  }
}

void time_fields(const DevMesh& m, const DevWindow& w, double4_32a* vt, cudaStream_t s) {
  if (w.nslots <= 0 || m.nnodes <= 0) return;
  k_time_fields<<<nblk(m.nnodes, 256), 256, 0, s>>>(w, m.nnodes, vt);
}

__global__ void k_pack_frame(const double* uvw, double4_32a* out, long n) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = make_double4_32a(uvw[3 * i], uvw[3 * i + 1], uvw[3 * i + 2], 0.0);
}

void pack_frame(const double* uvw, double4_32a* out, long n, cudaStream_t s) {
  k_pack_frame<<<nblk(n, 256), 256, 0, s>>>(uvw, out, n);
}

// ====================================================== seed location chain
//
// ompVC locates seeds one after another, each neighbour walk starting from
// the element found for an earlier seed (its "guess").  The walk's answer
// depends on the guess only for seeds within TINY of a shared face, so the
// chain is solved as a fixed point: start from the lowest-id containing
// element of every seed (bucketed global search), derive every seed's guess
// from the current answers with the reference's rules, redo every seed's
// walk from that guess in parallel, and repeat until nothing changes.  If
// the answers for seeds 0..m-1 equal the serial ones, the guess and hence the
// answer for seed m do too, so each round fixes at least the first
// difference and the fixed point is the serial result.

struct ChainDev {
  const double* X;
  const int* left0;
  const int* R0;   // global-search answer of every seed (FTLE chunks: of the marked seeds)
  const int* U;    // 1: R0 is the only element holding the seed (see k_global_unique)
  int* R;          // current answers
  int* Rn;         // next answers
  int* g;          // guess of every seed
  int* gprev;      // guesses of the previous round (null in the first round)
  int* planeexit;  // kind 0: the guess a plane leaves to the next, -1 none found
  int* planestart; // kind 0: the guess at the start of each plane
  int* planetarget;// kind 0 chunks: the seed whose answer is the plane's exit
  int* chunk_last; // rounds: last found seed of each block of 1024
  int* chunk_carry;
  int n, nplanes, plane, nchunks;
  int res[3];
  int kind, lsc, seed, pstar, init_guess;
};

// The kind 0 guess (ompVC/ftle.c:467-601, as its braces nest): the running
// guess is the last element found, across the rows of a plane as within
// them (jguess is taken up only after the j loop); at the end of a plane it
// becomes the first element found in the plane's last row (jguess), if any.
// iguess is taken up after the i loop, when no seed is left.

// Rounds: the guess each plane leaves, from the current answers.
__global__ void k_chain_plane_exit(ChainDev c) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.nplanes) return;
  const long base = (long)i * c.plane, last_row = base + (long)(c.res[1] - 1) * c.res[2];
  int e = -1;
  for (int k = 0; k < c.res[2] && e < 0; k++) e = c.R[last_row + k];
  for (long p = last_row - 1; p >= base && e < 0; p--) e = c.R[p];
  c.planeexit[i] = e;
}
__global__ void k_chain_planes(ChainDev c) {
  if (threadIdx.x || blockIdx.x) return;
  int G = c.init_guess;
  for (int i = 0; i < c.nplanes; i++) {
    c.planestart[i] = G;
    if (c.planeexit[i] >= 0) G = c.planeexit[i];
  }
}

// kinds 1 and 2 (ompVC/tracers.c:1156-1243, 1379-1524): the guess is the
// last element found before the seed in list order; kind 0 the same within
// a plane, else the plane's start.
__global__ void k_chain_chunk_last(ChainDev c) {
  __shared__ int best;
  if (threadIdx.x == 0) best = -1;
  __syncthreads();
  long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p < c.n && c.R[p] >= 0) atomicMax(&best, (int)p);
  __syncthreads();
  if (threadIdx.x == 0) c.chunk_last[blockIdx.x] = best;
}
__global__ void k_chain_carry(ChainDev c) {
  if (threadIdx.x || blockIdx.x) return;
  int run = -1;
  for (int b = 0; b < c.nchunks; b++) {
    c.chunk_carry[b] = run;
    if (c.chunk_last[b] >= 0) run = c.chunk_last[b];
  }
}
__global__ void k_chain_linear_guess(ChainDev c) {
  // exclusive max-scan of "index of a found seed" within the block
  __shared__ int warp_max[32];
  long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int v = (p < c.n && c.R[p] >= 0) ? (int)p : -1;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x = max(x, y);
  }
  if (lane == 31) warp_max[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int ws = lane < nw ? warp_max[lane] : -1;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, ws, o);
      if (lane >= o) ws = max(ws, y);
    }
    if (lane < nw) warp_max[lane] = ws;
  }
  __syncthreads();
  int before_warp = wid > 0 ? warp_max[wid - 1] : -1;
  int incl = max(x, before_warp);
  int excl_in_block = __shfl_up_sync(0xffffffffu, incl, 1);
  if (lane == 0) excl_in_block = before_warp;
  int last = max(excl_in_block, c.chunk_carry[blockIdx.x]);
  if (p >= c.n) return;
  if (c.kind == 0) {
    const long i = p / c.plane;
    c.g[p] = last >= i * c.plane ? c.R[last] : c.planestart[i];
  } else {
    c.g[p] = last >= 0 ? c.R[last] : c.init_guess;
  }
}

template <int DIMS>
__global__ void k_chain_eval(DevMesh m, ChainDev c, DevCounters* ctr) {
  long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
  int err = 0, changed = 0;
  if (p < c.n) {
    int r;
    if (c.left0[p]) r = -1;
    else if (p <= c.pstar) r = c.R0[p];
    else if (c.U && c.lsc && c.U[p]) r = c.R0[p];  // every walk ends there (k_global_unique)
    else if (c.gprev && c.gprev[p] == c.g[p]) r = c.R[p];  // same guess, same walk
    else {
      double x[3] = {c.X[3 * p], c.X[3 * p + 1], c.X[3 * p + 2]};
      r = locate_once<DIMS>(m, x, c.g[p], err);
      if (r < 0 && c.kind != 1) r = locate_once<DIMS>(m, x, c.seed, err);
      if (r < 0 && c.lsc) r = c.R0[p];
    }
    c.Rn[p] = r;
    changed = r != c.R[p];
  }
  int any = __reduce_or_sync(0xffffffffu, changed);
  int e = __reduce_or_sync(0xffffffffu, err);
  if ((threadIdx.x & 31) == 0) {
    if (any) atomicOr(&ctr->changed, 1);
    if (e) atomicOr(&ctr->status, e);
  }
}

// The FTLE chain (kind 0) with a centre element and LocalSearchChecking,
// solved in its own order instead of by rounds: ompVC's answer for a seed
// depends on its guess only when the seed lies within TINY of a shared face,
// and on such seeds (grid points on the cube's edges, for example) the
// rounds of the fixed point advance one seed at a time.  With
// LocalSearchChecking a seed the global search finds in one element alone
// has that element as its answer whatever its guess, and whether a seed is
// found at all does not depend on its guess (the global search settles it).
// Each plane's seeds are cut into chunks of CHAIN_CHUNK in loop order; the
// seeds that end a chunk, those of each plane's last row and each row's
// first are tested (k_chain_marks).  A chunk after a uniquely held seed starts from that
// seed's element; one after any other seed is taken on by the thread of the
// chunk before it, which goes on past its end.  The guess a plane leaves is
// the answer of one seed (the first found in its last row, or the plane's
// last found seed), worked out from the nearest uniquely held seed before
// it; only when the plane holds none before it does the plane's start enter,
// and the serial pass over the planes then walks that plane from its start.
// Every seed is evaluated with exactly the guess the serial loop holds.
constexpr int CHAIN_CHUNK = 16;

// One seed with the given guess (ompVC/ftle.c:520-597): a walk from the
// guess, then from the centre seed's element, then the global search when
// LocalSearchChecking is set.
template <int DIMS>
__device__ __forceinline__ int chain_one(const DevMesh& m, const BucketGrid& g, const ChainDev& c, long p,
                                         int guess, int& err) {
  if (c.left0[p]) return -1;
  if (c.U[p]) return c.R0[p];  // every walk ends there
  const double x[3] = {c.X[3 * p], c.X[3 * p + 1], c.X[3 * p + 2]};
  int r = locate_once<DIMS>(m, x, guess, err);
  if (r < 0) r = locate_once<DIMS>(m, x, c.seed, err);
  if (r < 0) r = global_find<DIMS>(m, g, x);
  return r;
}

// first: lowest-id element holding x among the bucket's candidates; the
// return value counts them up to 2
template <int DIMS>
__device__ __forceinline__ int holders(const DevMesh& m, const BucketGrid& g, const double x[3], int& first) {
  first = -1;
  int cc[3];
  for (int a = 0; a < 3; a++) {
    if (a == 2 && DIMS == 2) { cc[a] = 0; continue; }
    double f = (x[a] - g.lo[a]) * g.inv[a];
    if (!(f >= 0.0) || f >= (double)g.n[a]) return 0;
    cc[a] = min(g.n[a] - 1, (int)f);
  }
  const long cell = ((long)cc[2] * g.n[1] + cc[1]) * g.n[0] + cc[0];
  const int b0 = __ldg(g.start + cell), e0 = __ldg(g.start + cell + 1);
  const PosF P = pos_f32(x);
  int hits = 0;
  for (int q = b0; q < e0 && hits < 2; q++) {
    const int el = __ldg(g.ids + q);
    const int qs = quick_hop<DIMS>(m, el, P);
    if (qs >= 0) continue;
    if (qs == -2 || contains<DIMS>(m, el, x)) {
      if (!hits) first = el;
      hits++;
    }
  }
  return hits;
}

// R0 and U for the seeds that end a chunk of their plane, the seeds of each
// plane's last row and the first seed of every row; every other seed gets
// U = 0 and R0 = -1.  A row's first seed is walked to from the previous
// row's last, across the whole grid; held by one element, it needs no walk.
template <int DIMS>
__global__ void k_chain_marks(DevMesh m, BucketGrid g, ChainDev c) {
  const long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= c.n) return;
  const int q = (int)(p % c.plane);
  const bool mark = (q + 1) % CHAIN_CHUNK == 0 || q + 1 == c.plane || q >= (c.res[1] - 1) * c.res[2] ||
                    q % c.res[2] == 0;
  int first = -1, hits = 0;
  if (mark && !c.left0[p]) {
    const double x[3] = {c.X[3 * p], c.X[3 * p + 1], c.X[3 * p + 2]};
    hits = holders<DIMS>(m, g, x, first);
  }
  const_cast<int*>(c.R0)[p] = first;
  const_cast<int*>(c.U)[p] = hits == 1;
}

// The guess plane i leaves, where it does not depend on the plane's start:
// planeexit = that element (-1: no seed of the plane is found, the guess
// passes through), planetarget = the seed it is the answer of; planeexit =
// -2 when the plane holds no uniquely held seed before the target.
template <int DIMS>
__global__ void k_chain_exits(DevMesh m, BucketGrid g, ChainDev c, DevCounters* ctr) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.nplanes) return;
  const long base = (long)i * c.plane, last_row = base + (long)(c.res[1] - 1) * c.res[2];
  long t = -1;
  for (int k = 0; k < c.res[2] && t < 0; k++)
    if (!c.left0[last_row + k] && c.R0[last_row + k] >= 0) t = last_row + k;
  for (long p = last_row - 1; p >= base && t < 0; p--) {
    if (c.left0[p]) continue;
    int first = c.R0[p];
    if (first < 0) {
      const double x[3] = {c.X[3 * p], c.X[3 * p + 1], c.X[3 * p + 2]};
      holders<DIMS>(m, g, x, first);
    }
    if (first >= 0) t = p;
  }
  c.planetarget[i] = (int)t;
  if (t < 0) { c.planeexit[i] = -1; return; }
  long a = t - 1;
  if (!c.U[t])
    while (a >= base && !c.U[a]) a--;
  if (!c.U[t] && a < base) { c.planeexit[i] = -2; return; }
  int err = 0, G = c.U[t] ? c.R0[t] : c.R0[a];
  if (!c.U[t])
    for (long p = a + 1; p <= t; p++) {
      const int r = chain_one<DIMS>(m, g, c, p, G, err);
      if (r >= 0) G = r;
    }
  c.planeexit[i] = G;
  if (err) atomicOr(&ctr->status, err);
}

// The planes in order: each plane's start, walking a plane from its start
// where its exit depends on it.
template <int DIMS>
__global__ void k_chain_plane_starts(DevMesh m, BucketGrid g, ChainDev c, DevCounters* ctr) {
  if (threadIdx.x || blockIdx.x) return;
  int err = 0, G = c.init_guess;
  for (int i = 0; i < c.nplanes; i++) {
    c.planestart[i] = G;
    int e = c.planeexit[i];
    if (e == -2) {
      for (long p = (long)i * c.plane; p <= c.planetarget[i]; p++) {
        const int r = chain_one<DIMS>(m, g, c, p, G, err);
        if (r >= 0) G = r;
      }
    } else if (e >= 0) {
      G = e;
    }
  }
  if (err) atomicOr(&ctr->status, err);
}

// One thread per (plane, chunk): the chunk's seeds from its starting guess,
// on into the next chunks until one starts after a uniquely held seed.
template <int DIMS>
__global__ void k_chain_points(DevMesh m, BucketGrid g, ChainDev c, int* eid, DevCounters* ctr) {
  const int nch = (c.plane + CHAIN_CHUNK - 1) / CHAIN_CHUNK;
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)c.nplanes * nch) return;
  const long i = t / nch;
  const int ch = (int)(t % nch), start = ch * CHAIN_CHUNK;
  const long base = i * c.plane;
  int cur;
  if (ch == 0) cur = c.planestart[i];
  else if (c.U[base + start - 1]) cur = c.R0[base + start - 1];
  else return;  // the chunk before goes on into this one
  int err = 0;
  for (int q = start; q < c.plane; q++) {
    if (q > start && q % CHAIN_CHUNK == 0 && c.U[base + q - 1]) break;  // that chunk's own thread
    const long p = base + q;
    const int r = chain_one<DIMS>(m, g, c, p, cur, err);
    eid[p] = r;
    if (r >= 0) cur = r;
  }
  if (err) atomicOr(&ctr->status, err);
}

__global__ void k_first_found(int n, const int* left0, const int* R0, int* out) {
  long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p < n && !left0[p] && R0[p] >= 0) atomicMin(out, (int)p);
}

size_t chain_words(const ChainArgs& a) {
  const size_t planes = a.kind == 0 ? (size_t)a.res[0] : 0;
  return 6 * (size_t)a.n + 3 * (planes + 1) + 2 * ((size_t)a.n / 1024 + 2) + 16;
}

int locate_chain(const DevMesh& m, const BucketGrid& g, const ChainArgs& a, const double* X,
                 const int* left0, int* eid, int* work, DevCounters* ctr, cudaStream_t s) {
  ChainDev c;
  int n = a.n;
  c.X = X;
  c.left0 = left0;
  c.n = n;
  c.kind = a.kind;
  c.lsc = a.lsc;
  c.res[0] = a.res[0];
  c.res[1] = a.res[1];
  c.res[2] = a.res[2];
  c.nplanes = a.kind == 0 ? a.res[0] : 0;
  c.plane = a.kind == 0 ? a.res[1] * a.res[2] : 1;
  c.nchunks = nblk(n, 1024);
  int* w = work;
  int* R0 = w; w += n;
  int* U = w; w += n;
  c.R = w; w += n;
  c.Rn = w; w += n;
  c.g = w; w += n;
  int* gother = w; w += n;
  c.gprev = nullptr;
  c.planeexit = w; w += c.nplanes + 1;
  c.planestart = w; w += c.nplanes + 1;
  c.planetarget = w; w += c.nplanes + 1;
  c.chunk_last = w; w += c.nchunks + 1;
  c.chunk_carry = w; w += c.nchunks + 1;
  int* d_first = w; w += 1;
  c.R0 = R0;
  c.U = U;
  if (a.kind == 0 && a.center_eid >= 0 && a.lsc) {
    c.seed = a.center_eid;
    c.pstar = -1;
    c.init_guess = a.center_eid;
    const long nch = (long)c.nplanes * ((c.plane + CHAIN_CHUNK - 1) / CHAIN_CHUNK);
    if (m.dims == 3) {
      k_chain_marks<3><<<nblk(n, 128), 128, 0, s>>>(m, g, c);
      k_chain_exits<3><<<nblk(c.nplanes, 32), 32, 0, s>>>(m, g, c, ctr);
      k_chain_plane_starts<3><<<1, 32, 0, s>>>(m, g, c, ctr);
      k_chain_points<3><<<nblk(nch, 64), 64, 0, s>>>(m, g, c, eid, ctr);
    } else {
      k_chain_marks<2><<<nblk(n, 128), 128, 0, s>>>(m, g, c);
      k_chain_exits<2><<<nblk(c.nplanes, 32), 32, 0, s>>>(m, g, c, ctr);
      k_chain_plane_starts<2><<<1, 32, 0, s>>>(m, g, c, ctr);
      k_chain_points<2><<<nblk(nch, 64), 64, 0, s>>>(m, g, c, eid, ctr);
    }
    int status = 0;
    cudaMemcpyAsync(&status, &ctr->status, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess || status) return -1;
    return 0;
  }
  // every seed's global-search answer and whether it is the only element
  // holding it: such seeds' answers do not depend on their guesses (with
  // LocalSearchChecking), which leaves the rounds' walks to the few seeds on
  // shared faces (a seed list's consecutive seeds can lie far apart)
  if (m.dims == 3) k_global_unique<3><<<nblk(n, 128), 128, 0, s>>>(m, g, n, X, left0, R0, U);
  else k_global_unique<2><<<nblk(n, 128), 128, 0, s>>>(m, g, n, X, left0, R0, U);
  // first seed found by the global search: the chain's start when no centre
  // element is known (and always for a tracer list)
  int big = 0x7fffffff, first = big;
  cudaMemcpyAsync(d_first, &big, sizeof(int), cudaMemcpyHostToDevice, s);
  k_first_found<<<nblk(n, 256), 256, 0, s>>>(n, left0, R0, d_first);
  cudaMemcpyAsync(&first, d_first, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return -1;
  if (a.kind != 1 && a.center_eid >= 0) {
    c.seed = a.center_eid;
    c.pstar = -1;
    c.init_guess = a.center_eid;
  } else if (first == big) {  // nothing inside the mesh
    cudaMemcpyAsync(eid, R0, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice, s);
    return 0;
  } else {
    int sv = 0;
    cudaMemcpyAsync(&sv, R0 + first, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return -1;
    c.seed = sv;
    c.pstar = first;
    c.init_guess = -1;
  }
  cudaMemcpyAsync(c.R, R0, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice, s);
  int rounds = 0;
  for (;;) {
    rounds++;
    if (a.kind == 0) {
      k_chain_plane_exit<<<nblk(c.nplanes, 128), 128, 0, s>>>(c);
      k_chain_planes<<<1, 32, 0, s>>>(c);
    }
    k_chain_chunk_last<<<c.nchunks, 1024, 0, s>>>(c);
    k_chain_carry<<<1, 32, 0, s>>>(c);
    k_chain_linear_guess<<<c.nchunks, 1024, 0, s>>>(c);
    cudaMemsetAsync(&ctr->changed, 0, sizeof(int), s);
    if (m.dims == 3) k_chain_eval<3><<<nblk(n, 128), 128, 0, s>>>(m, c, ctr);
    else k_chain_eval<2><<<nblk(n, 128), 128, 0, s>>>(m, c, ctr);
    int changed = 0, status = 0;
    cudaMemcpyAsync(&changed, &ctr->changed, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&status, &ctr->status, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess || status) return -1;
    int* t = c.R;
    c.R = c.Rn;
    c.Rn = t;
    // next round writes its guesses over the older array
    int* gp = c.g;
    c.g = c.gprev ? c.gprev : gother;
    c.gprev = gp;
    if (!changed || rounds > n + 1) break;
  }
  cudaMemcpyAsync(eid, c.R, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice, s);
  return rounds;
}

// ================================================================ FTLE

__global__ void k_ftle_seed(DevMesh m, FtleDev f, double xmin, double ymin, double zmin, int* left0) {
  long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= f.n) return;
  int k = (int)(p % f.zr), j = (int)((p / f.zr) % f.yr), i = (int)(p / ((long)f.zr * f.yr));
  // InitializeFTLEArray, ompVC/ftle.c:410-423
  double x[3] = {xmin + i * f.dx, ymin + j * f.dy, zmin + k * f.dz};
  f.X[3 * p] = x[0];
  f.X[3 * p + 1] = x[1];
  f.X[3 * p + 2] = x[2];
  f.V[3 * p] = f.V[3 * p + 1] = f.V[3 * p + 2] = 0.0;
  f.ftT[p] = 0.0;
  f.ftN[p] = 0.0;
  f.have[p] = 0;
  f.left[p] = 0;
  f.ldt[p] = 0.0;
  f.eid[p] = -1;
  left0[p] = outside_domain(m, x);
}

void ftle_seed_grid(const DevMesh& m, const FtleDev& f, double xmin, double ymin, double zmin,
                    int* left0, cudaStream_t s) {
  k_ftle_seed<<<nblk(f.n, 256), 256, 0, s>>>(m, f, xmin, ymin, zmin, left0);
}

// Points outside the domain or the mesh: FTLE -1, and no FTLE is computed
// for them or their six neighbours (ompVC/ftle.c:429-449, 476-496).  The
// left flag marks them on entry.
__global__ void k_ftle_outside(FtleDev f) {
  long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= f.n || !f.left[p]) return;
  int YZ = f.yr * f.zr;
  int k = (int)(p % f.zr), j = (int)((p / f.zr) % f.yr), i = (int)(p / YZ);
  f.ldt[p] = -1.0;
  f.ftT[p] = -1.0;
  f.ftN[p] = -1.0;
  f.have[p] = 1;
  if (i > 0) f.have[p - YZ] = 1;
  if (i < f.xr - 1) f.have[p + YZ] = 1;
  if (j > 0) f.have[p - f.zr] = 1;
  if (j < f.yr - 1) f.have[p + f.zr] = 1;
  if (k > 0) f.have[p - 1] = 1;
  if (k < f.zr - 1) f.have[p + 1] = 1;
}

void ftle_mark_outside(const FtleDev& f, cudaStream_t s) {
  k_ftle_outside<<<nblk(f.n, 256), 256, 0, s>>>(f);
}

__global__ void k_ftle_init_marks(FtleDev f, const int* left0, int unstructured) {
  long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= f.n) return;
  f.left[p] = left0[p] || (unstructured && f.eid[p] < 0);
}

void ftle_init_marks(const DevMesh& m, const FtleDev& f, const int* left0, cudaStream_t s) {
  k_ftle_init_marks<<<nblk(f.n, 256), 256, 0, s>>>(f, left0, m.mesh_type == 1);
}

// Pass 2a: the trigger of every point without an FTLE value is the exiting
// member of {q} + 6 neighbours with the lowest linear index -- the exit whose
// GetFTLEForPointEarly calls (ompVC/ftle.c:130-152) reach q first.
__global__ void k_ftle_triggers(FtleDev f, DevCounters* ctr) {
  long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
  long trig = -1;
  if (q < f.n && !f.have[q]) {
    int YZ = f.yr * f.zr, zr = f.zr;
    int k = (int)(q % zr), j = (int)((q / zr) % f.yr), i = (int)(q / YZ);
    long cand[7] = {i > 0 ? q - YZ : -1, j > 0 ? q - zr : -1, k > 0 ? q - 1 : -1, q,
                    k < zr - 1 ? q + 1 : -1, j < f.yr - 1 ? q + zr : -1, i < f.xr - 1 ? q + YZ : -1};
#pragma unroll
    for (int c = 0; c < 7; c++)
      if (cand[c] >= 0 && (f.flag[cand[c]] & 2)) {
        trig = cand[c];
        break;
      }
  }
  // warp-aggregated append keeps a warp's served points adjacent in the list
  unsigned b = __ballot_sync(0xffffffffu, trig >= 0);
  if (!b) return;
  int lane = threadIdx.x & 31, base = 0;
  if (lane == 0) base = atomicAdd(&ctr->count, __popc(b));
  base = __shfl_sync(0xffffffffu, base, 0);
  if (trig < 0) return;
  int slot = base + __popc(b & ((1u << lane) - 1u));
  f.served[slot] = (int)q;
  f.trig[slot] = (int)trig;
}

void ftle_triggers(const FtleDev& f, DevCounters* ctr, bool cleared, cudaStream_t s) {
  if (!cleared) cudaMemsetAsync(&ctr->count, 0, FVC_EARLY_COUNTERS_BYTES, s);
  k_ftle_triggers<<<nblk(f.n, 256), 256, 0, s>>>(f, ctr);
}

// UpdateFTLELocations and the per-point writes of ompVC/ftle.c:155-169, 175.
// Every point's flag is cleared for the next interval, and with nlive the
// next interval's live list is built here (the points compact_live would
// select), appended a block at a time.  Its threads then take the points in
// bricks of 32 (2 x 4 x 4 in i, j, k; 4 x 8 in 2D), so that a warp of the
// main pass, which takes 32 entries of the list, advects a compact piece of
// the grid whose walks share elements.
struct Bricks {
  int bi, bj, bk, nj, nk;
  long count;  // threads: bricks x 32
};

static Bricks bricks_of(const FtleDev& f) {
  Bricks b;
  b.bk = f.zr > 1 ? 4 : 1;
  b.bi = f.zr > 1 ? 2 : 4;
  b.bj = 32 / (b.bi * b.bk);
  b.nj = (f.yr + b.bj - 1) / b.bj;
  b.nk = (f.zr + b.bk - 1) / b.bk;
  b.count = 32L * ((f.xr + b.bi - 1) / b.bi) * b.nj * b.nk;
  return b;
}

__device__ __forceinline__ long brick_point(const FtleDev& f, const Bricks& b, long t) {
  const long T = t >> 5;
  const int l = (int)(t & 31);
  const long Tk = T % b.nk, Tj = (T / b.nk) % b.nj, Ti = T / ((long)b.nk * b.nj);
  const long i = Ti * b.bi + l / (b.bj * b.bk), j = Tj * b.bj + (l / b.bk) % b.bj, k = Tk * b.bk + l % b.bk;
  if (i >= f.xr || j >= f.yr || k >= f.zr) return -1;
  return (i * f.yr + j) * f.zr + k;
}

// update 0: only the live list (and the cleared flags) for the state as it
// stands, the interval's first step after a launch or a host state change.
// With nfall, the first threads first solve the early-FTLE points the
// closed-form eigenvalue left (k_ftle_early_jacobi's work, a few hundred
// points; the other blocks' updates run meanwhile).
__global__ void __launch_bounds__(256) k_ftle_update(FtleDev f, Bricks br, int update, int extrapolate,
                                                     int unstructured, int* nlive, const int* nfall, int dims) {
  __shared__ int warp_off[8];
  __shared__ int block_base;
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (nfall) {
    const long nf = *(volatile const int*)nfall;
    const int* fall = reinterpret_cast<const int*>(f.tasks);
    for (long i = t; i < nf; i += (long)gridDim.x * blockDim.x) {
      if (dims == 3) early_final_one<3>(f, fall[i], true);
      else early_final_one<2>(f, fall[i], true);
    }
  }
  const long p = nlive ? (t < br.count ? brick_point(f, br, t) : -1) : t;
  bool live = false;
  if (p >= 0 && p < f.n) {
    const unsigned char fl = update ? f.flag[p] : 1;
    int left = f.left[p];
    if (update && (fl & 1)) {
      if (fl & 2) {
        left = 1;
        f.left[p] = 1;
      } else {
        f.X[3 * p] = f.Xn[3 * p];
        f.X[3 * p + 1] = f.Xn[3 * p + 1];
        f.X[3 * p + 2] = f.Xn[3 * p + 2];
        if (extrapolate) {
          f.V[3 * p] = f.Vn[3 * p];
          f.V[3 * p + 1] = f.Vn[3 * p + 1];
          f.V[3 * p + 2] = f.Vn[3 * p + 2];
          left = (fl & 4) ? 1 : 0;
          f.left[p] = left;
        }
        if (unstructured) f.eid[p] = f.en[p];
      }
    }
    if (fl) f.flag[p] = 0;
    live = nlive && f.ldt[p] > -FVC_TINY && (!left || extrapolate);
  }
  if (!nlive) return;
  const unsigned b = __ballot_sync(0xffffffffu, live);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) warp_off[wid] = __popc(b);
  __syncthreads();
  if (threadIdx.x == 0) {
    int c = 0;
    for (int k = 0; k < 8; k++) {
      const int v = warp_off[k];
      warp_off[k] = c;
      c += v;
    }
    block_base = c ? atomicAdd(nlive, c) : 0;
  }
  __syncthreads();
  if (live) f.live[block_base + warp_off[wid] + __popc(b & ((1u << lane) - 1u))] = (int)p;
}

void ftle_update(const DevMesh& m, const DevInteg& in, const FtleDev& f, DevCounters* ctr, cudaStream_t s) {
  const Bricks br = bricks_of(f);
  // the live count and the next interval's work cursors (adjacent)
  if (ctr) cudaMemsetAsync(&ctr->nlive, 0, sizeof(int) + sizeof(ctr->cur), s);
  k_ftle_update<<<nblk(ctr ? br.count : f.n, 256), 256, 0, s>>>(f, br, 1, in.extrapolate, m.mesh_type == 1,
                                                                 ctr ? &ctr->nlive : nullptr,
                                                                 ctr ? &ctr->nfall : nullptr, m.dims);
}

void ftle_live(const DevInteg& in, const FtleDev& f, DevCounters* ctr, cudaStream_t s) {
  const Bricks br = bricks_of(f);
  cudaMemsetAsync(&ctr->nlive, 0, sizeof(int) + sizeof(ctr->cur), s);
  k_ftle_update<<<nblk(br.count, 256), 256, 0, s>>>(f, br, 0, in.extrapolate, 0, &ctr->nlive, nullptr, 0);
}

// GetFTLEForPoint (ompVC/ftle.c:1050-1203) for points without a value, and
// the output transpose to k, j, i order (ompVC/ftle.c:1304-1315).
__global__ void k_ftle_final(FtleDev f, int dims, double int_t) {
  long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= f.n) return;
  int YZ = f.yr * f.zr, zr = f.zr;
  int k = (int)(q % zr), j = (int)((q / zr) % f.yr), i = (int)(q / YZ);
  double wT = f.ftT[q], wN = f.ftN[q];
  if (!f.have[q]) {
    if (int_t < FVC_TINY) {
      wT = 0.0;
      wN = 0.0;
    } else {
      const double* X = f.X;
      const double *L, *R, *B, *T, *Bk, *F;
      double fx, fy, fz;
      if (i == 0) { L = X + 3 * q; R = X + 3 * (q + YZ); fx = 1.0; }
      else if (i == f.xr - 1) { L = X + 3 * (q - YZ); R = X + 3 * q; fx = 1.0; }
      else { L = X + 3 * (q - YZ); R = X + 3 * (q + YZ); fx = 2.0; }
      if (j == 0) { B = X + 3 * q; T = X + 3 * (q + zr); fy = 1.0; }
      else if (j == f.yr - 1) { B = X + 3 * (q - zr); T = X + 3 * q; fy = 1.0; }
      else { B = X + 3 * (q - zr); T = X + 3 * (q + zr); fy = 2.0; }
      if (dims == 3) {
        if (k == 0) { Bk = X + 3 * q; F = X + 3 * (q + 1); fz = 1.0; }
        else if (k == zr - 1) { Bk = X + 3 * (q - 1); F = X + 3 * q; fz = 1.0; }
        else { Bk = X + 3 * (q - 1); F = X + 3 * (q + 1); fz = 2.0; }
      } else { Bk = F = X + 3 * q; fz = 1.0; }
      const double lm1 = stencil_lambda_m1(dims, L, R, B, T, Bk, F, fx, fy, fz, f.dx, f.dy, f.dz);
      if (lm1 > -FVC_TINY) {
        wN = 0.5 * log1p(lm1);
        wT = wN / int_t;
      } else {
        wT = 0.0;
        wN = 0.0;
      }
    }
    f.ftT[q] = wT;
    f.ftN[q] = wN;
  }
  long o = ((long)k * f.yr + j) * f.xr + i;
  f.out[o] = wT;
  f.out[f.n + o] = wN;
}

void ftle_final(const FtleDev& f, int dims, double int_t, cudaStream_t s) {
  k_ftle_final<<<nblk(f.n, 128), 128, 0, s>>>(f, dims, int_t);
}

// ============================================================== tracers

// LeftDomainTime of freshly located seeds: -1 outside, 0 inside
// (ompVC/tracers.c:1246-1249).
__global__ void k_tracer_ldt(TracerDev t) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= t.n) return;
  t.ldt[i] = t.left[i] ? -1.0 : 0.0;
  t.V[3 * i] = t.V[3 * i + 1] = t.V[3 * i + 2] = 0.0;
}

void tracer_init_ldt(const TracerDev& t, cudaStream_t s) {
  if (t.n > 0) k_tracer_ldt<<<nblk(t.n, 256), 256, 0, s>>>(t);
}

// ReadInTraceMesh (chain 0, ompVC/tracers.c:1246-1249): LeftDomainTime -1 for
// every point left out.  GenerateTracerMesh (chain 1, tracers.c:1353-1466)
// sets -1 only for points inside the bounding box that no element holds and
// leaves the rest at 0.
__global__ void k_tracer_init_marks(TracerDev t, const int* left0, int unstructured, int chain) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= t.n) return;
  int unplaced = unstructured && !left0[i] && t.eid[i] < 0;
  int left = left0[i] || unplaced;
  t.left[i] = left;
  t.ldt[i] = chain == 0 ? (left ? -1.0 : 0.0) : (unplaced ? -1.0 : 0.0);
  if (!unstructured || left) t.eid[i] = -1;
  t.V[3 * i] = t.V[3 * i + 1] = t.V[3 * i + 2] = 0.0;
}

void tracer_init_marks(const DevMesh& m, const TracerDev& t, const int* left0, int chain_kind,
                       cudaStream_t s) {
  if (t.n > 0) k_tracer_init_marks<<<nblk(t.n, 256), 256, 0, s>>>(t, left0, m.mesh_type == 1, chain_kind);
}

// Output selection of ompVC/tracers.c:247: compaction in seed order with
// warp ballots; block counts, a scan of them, then the scatter.
__device__ __forceinline__ bool tracer_selected(const TracerDev& t, long i, int always) {
  return i < t.n && t.ldt[i] > -FVC_TINY && (!t.left[i] || always);
}

__global__ void k_compact_count(TracerDev t, int always) {
  __shared__ int warp_cnt[32];
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned b = __ballot_sync(0xffffffffu, tracer_selected(t, i, always));
  if ((threadIdx.x & 31) == 0) warp_cnt[threadIdx.x >> 5] = __popc(b);
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) s += warp_cnt[k];
    t.block_cnt[blockIdx.x] = s;
  }
}

__global__ void k_compact_scatter(TracerDev t, int always, const int* block_off) {
  __shared__ int warp_off[32];
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  bool sel = tracer_selected(t, i, always);
  unsigned b = __ballot_sync(0xffffffffu, sel);
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) warp_off[wid] = __popc(b);
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) {
      int c = warp_off[k];
      warp_off[k] = s;
      s += c;
    }
  }
  __syncthreads();
  if (sel) {
    long o = (long)block_off[blockIdx.x] + warp_off[wid] + __popc(b & ((1u << lane) - 1u));
    t.outX[3 * o] = t.X[3 * i];
    t.outX[3 * o + 1] = t.X[3 * i + 1];
    t.outX[3 * o + 2] = t.X[3 * i + 2];
  }
}

__global__ void k_copy_count(const int* src, int* dst) { *dst = *src; }

// The scatter with each block's offset summed from the block counts before
// it (no scan launches; for up to COMPACT_DIRECT_BLOCKS blocks, a few
// thousand L2 reads a block); the last block writes the total.  unpack: the
// mixed form's (X, c) pairs are written as FP64 positions X - c (the same
// arithmetic as k_unpack_pairs).
constexpr int COMPACT_DIRECT_BLOCKS = 4096;
__global__ void __launch_bounds__(1024) k_compact_scatter_direct(TracerDev t, int always, int unpack, int* count) {
  __shared__ int warp_off[32];
  __shared__ long long red[32];
  __shared__ long long block_off;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  long long part = 0;
  for (int b = threadIdx.x; b < (int)blockIdx.x; b += blockDim.x) part += t.block_cnt[b];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  if (lane == 0) red[wid] = part;
  __syncthreads();
  if (threadIdx.x == 0) {
    long long a = 0;
    for (int k = 0; k < nw; k++) a += red[k];
    block_off = a;
  }
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  bool sel = tracer_selected(t, i, always);
  unsigned b = __ballot_sync(0xffffffffu, sel);
  if (lane == 0) warp_off[wid] = __popc(b);
  __syncthreads();
  if (threadIdx.x == 0) {
    int c = 0;
    for (int k = 0; k < nw; k++) {
      int v = warp_off[k];
      warp_off[k] = c;
      c += v;
    }
    if (blockIdx.x == gridDim.x - 1) *count = (int)(block_off + c);
  }
  __syncthreads();
  if (sel) {
    long o = (long)block_off + warp_off[wid] + __popc(b & ((1u << lane) - 1u));
#pragma unroll
    for (int a = 0; a < 3; a++)
      t.outX[3 * o + a] = unpack ? join_pos(reinterpret_cast<const float2*>(t.X)[3 * i + a]) : t.X[3 * i + a];
  }
}

// Live-point compaction: warp ballots give each lane its rank among the
// selected lanes; block counts are scanned into offsets so the list keeps the
// points' order (neighbouring points stay in the same warp).
__device__ __forceinline__ bool is_live(long i, int n, const double* ldt, const int* left, int extrap) {
  return i < n && ldt[i] > -FVC_TINY && (!left[i] || extrap);
}

__global__ void k_live_count(int n, const double* ldt, const int* left, int extrap, int* block_cnt) {
  __shared__ int warp_cnt[32];
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned b = __ballot_sync(0xffffffffu, is_live(i, n, ldt, left, extrap));
  if ((threadIdx.x & 31) == 0) warp_cnt[threadIdx.x >> 5] = __popc(b);
  __syncthreads();
  if (threadIdx.x == 0) {
    int c = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) c += warp_cnt[k];
    block_cnt[blockIdx.x] = c;
  }
}

__global__ void k_live_scatter(int n, const double* ldt, const int* left, int extrap, const int* block_off,
                               int* live, unsigned char* flag, DevCounters* ctr) {
  __shared__ int warp_off[32];
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  bool sel = is_live(i, n, ldt, left, extrap);
  unsigned b = __ballot_sync(0xffffffffu, sel);
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) warp_off[wid] = __popc(b);
  __syncthreads();
  if (threadIdx.x == 0) {
    int c = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) {
      int v = warp_off[k];
      warp_off[k] = c;
      c += v;
    }
  }
  __syncthreads();
  if (i < n && flag) flag[i] = 0;
  if (sel) live[block_off[blockIdx.x] + warp_off[wid] + __popc(b & ((1u << lane) - 1u))] = (int)i;
  // the live count, and the work cursors of the persistent launch that
  // takes the list next start at 0 (calls may be queued back to back on
  // the same counters)
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x < 5) {
    if (threadIdx.x == 0) ctr->nlive = block_off[gridDim.x];
    else ctr->cur[threadIdx.x - 1] = 0;
  }
}

void compact_live(int n, const double* ldt, const int* left, int extrapolate, int* live,
                  unsigned char* flag, int* block_cnt, DevCounters* ctr, cudaStream_t s) {
  if (n <= 0) {
    cudaMemsetAsync(&ctr->nlive, 0, sizeof(int) * 5, s);  // nlive and the cursors
    return;
  }
  unsigned nb = nblk(n, 1024);
  int* off = block_cnt + nb + 1;
  long long* tmp = reinterpret_cast<long long*>(block_cnt + ((2 * nb + 4) & ~1u));
  k_live_count<<<nb, 1024, 0, s>>>(n, ldt, left, extrapolate, block_cnt);
  exclusive_scan(block_cnt, off, (int)nb, tmp, s);
  k_live_scatter<<<nb, 1024, 0, s>>>(n, ldt, left, extrapolate, off, live, flag, ctr);
}

int tracer_compact(const TracerDev& t, int always, DevCounters* ctr, cudaStream_t s, bool unpack) {
  if (t.n <= 0) {
    cudaMemsetAsync(&ctr->count, 0, sizeof(int), s);
    return 0;
  }
  unsigned nb = nblk(t.n, 1024);
  k_compact_count<<<nb, 1024, 0, s>>>(t, always);
  if (nb <= (unsigned)COMPACT_DIRECT_BLOCKS) {
    k_compact_scatter_direct<<<nb, 1024, 0, s>>>(t, always, unpack ? 1 : 0, &ctr->count);
    return 2;
  }
  // block_cnt has room for nb + 1 offsets followed by the scan's block totals
  int* off = t.block_cnt + nb + 1;
  long long* tmp = reinterpret_cast<long long*>(t.block_cnt + ((2 * nb + 4) & ~1u));
  exclusive_scan(t.block_cnt, off, (int)nb, tmp, s);
  k_compact_scatter<<<nb, 1024, 0, s>>>(t, always, off);
  k_copy_count<<<1, 1, 0, s>>>(off + nb, &ctr->count);
  if (unpack) unpack_pairs_counted(t.outX, t.n, &ctr->count, s);
  return 5 + (unpack ? 1 : 0);
}


// ---------------------------------------------------- per-variant dispatch

#define FVC_VARIANT(m, CALL)                                          \
  do {                                                                \
    if ((m).prec) {                                                   \
      if ((m).dims == 2) VariantMx<2>::CALL; else VariantMx<3>::CALL; \
    } else if ((m).mesh_type == 0) {                                  \
      if ((m).dims == 2) Variant<2, 0>::CALL; else Variant<3, 0>::CALL; \
    } else {                                                          \
      if ((m).dims == 2) Variant<2, 1>::CALL; else Variant<3, 1>::CALL; \
    }                                                                 \
  } while (0)

void launch_advect(const DevMesh& m, const DevWindow& w, const DevInteg& in, int n, double* X,
                   double* V, int* eid, int* left, double* ldt, double t0, double t1,
                   DevCounters* ctr, cudaStream_t s) {
  if (n > 0) FVC_VARIANT(m, advect(m, w, in, n, X, V, eid, left, ldt, t0, t1, ctr, s));
}
void launch_velocity(const DevMesh& m, const DevWindow& w, int n, const double* X, int* eid,
                     int* left, double tq, double* out, DevCounters* ctr, cudaStream_t s) {
  if (n > 0) FVC_VARIANT(m, velocity(m, w, n, X, eid, left, tq, out, ctr, s));
}
void ftle_launch(const DevMesh& m, const DevWindow& w, const FtleDev& f, double t, DevCounters* ctr,
                 cudaStream_t s) {
  FVC_VARIANT(m, ftle_launch(m, w, f, t, ctr, s));
}
void ftle_pass1(const DevMesh& m, const DevWindow& w, const DevInteg& in, const FtleDev& f,
                double t1, double t2, DevCounters* ctr, cudaStream_t s) {
  FVC_VARIANT(m, ftle_pass1(m, w, in, f, t1, t2, ctr, s));
}
void ftle_early(const DevMesh& m, const DevWindow& w, const DevInteg& in, const FtleDev& f,
                double t1, DevCounters* ctr, bool jacobi, cudaStream_t s) {
  FVC_VARIANT(m, ftle_early(m, w, in, f, t1, ctr, jacobi, s));
}
void tracer_launch_vel(const DevMesh& m, const DevWindow& w, const TracerDev& t, double tq,
                       DevCounters* ctr, cudaStream_t s) {
  if (t.n > 0) FVC_VARIANT(m, tracer_launch(m, w, t, tq, ctr, s));
}
void tracer_advance(const DevMesh& m, const DevWindow& w, const DevInteg& in, const TracerDev& t,
                    double t1, double t2, DevCounters* ctr, cudaStream_t s) {
  if (t.n > 0) FVC_VARIANT(m, tracer_advance(m, w, in, t, t1, t2, ctr, s));
}

}  // namespace fvc
