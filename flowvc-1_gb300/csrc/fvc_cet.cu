// fvc_cet.cu -- tracer side analyses: exposure time (Trace_CETCompute,
// ompVC/exposuretime.c) and residence time (Trace_RTCompute,
// ompVC/residencetime.c), on unstructured meshes in the FP64 form.
#include "fvc_advect_impl.cuh"

namespace fvc {

// k_tracer_advance with the exposure-time hook after every accepted step
// (ompVC/integration.c:277-299, 427-447, 649-669).
template <int D>
__global__ void __launch_bounds__(128) k_tracer_advance_cet(DevMesh m, DevWindow w, DevInteg in, TracerDev t,
                                                           double t1, double t2, CetDev cet, DevCounters* ctr) {
  const long nlive = *(volatile int*)&ctr->nlive;
  unsigned steps = 0;
  int err = 0;
  for (long base = warp_grab(&ctr->cur[0]); base < nlive; base = warp_grab(&ctr->cur[0])) {
    const long idx = base + (threadIdx.x & 31);
    if (idx >= nlive) continue;
    long i = t.live[idx];
    Pt p;
    load_pt(p, i, t.X, t.V, t.eid, t.left, t.ldt);
    err |= advect<D, 1, true>(m, w, in, p, t1, t2, steps, &cet);
    t.X[3 * i] = p.X[0];
    t.X[3 * i + 1] = p.X[1];
    t.X[3 * i + 2] = p.X[2];
    t.V[3 * i] = p.V[0];
    t.V[3 * i + 1] = p.V[1];
    t.V[3 * i + 2] = p.V[2];
    t.eid[i] = p.eid;
    t.left[i] = p.left;
    t.ldt[i] = p.ldt;
  }
  flush_counters(&ctr->steps, &ctr->status, steps, err);
}

void tracer_advance_cet(const DevMesh& m, const DevWindow& w, const DevInteg& in, const TracerDev& t, double t1,
                        double t2, const CetDev& cet, DevCounters* ctr, cudaStream_t s) {
  if (t.n <= 0) return;
  if (m.dims == 3) {
    static const unsigned res = resident_blocks(k_tracer_advance_cet<3>, 128);
    k_tracer_advance_cet<3><<<capped(t.n, 128, res), 128, 0, s>>>(m, w, in, t, t1, t2, cet, ctr);
  } else {
    static const unsigned res = resident_blocks(k_tracer_advance_cet<2>, 128);
    k_tracer_advance_cet<2><<<capped(t.n, 128, res), 128, 0, s>>>(m, w, in, t, t1, t2, cet, ctr);
  }
}

// A release's first encounters: one for the element of every tracer inside
// the domain (ompVC/tracers.c:180-185).
__global__ void k_cet_release(TracerDev t, CetDev cet) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= t.n || t.left[i]) return;
  atomicAdd(cet.enc + t.eid[i], 1);
}

void cet_release(const TracerDev& t, const CetDev& cet, cudaStream_t s) {
  if (t.n > 0) k_cet_release<<<vblk(t.n, 256), 256, 0, s>>>(t, cet);
}

// OutputCET, ompVC/exposuretime.c:175-246: CET = sum / xc / ntracers and
// MET = sum / xc / encounters where sum > TINY, else 0.  In 3D the
// reference's xc is pow(vol, (1/3)) with the integer quotient 1/3 = 0, so
// xc = 1; in 2D xc = sqrt(triangle area).  out: CET then MET, nelem each.
template <int D>
__global__ void k_cet_results(DevMesh m, CetDev cet, double ntracers, double* out) {
  long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m.nelem) return;
  const double sum = cet.sum[e];
  double c = 0.0, mt = 0.0;
  if (sum > FVC_TINY) {
    double xc = 1.0;
    if (D == 2) {
      const int4 nd = m.elem[2 * e];
      const double4_32a p1 = m.nodes[nd.x], p2 = m.nodes[nd.y], p3 = m.nodes[nd.z];
      const double A0 = p2.x - p1.x, A1 = p2.y - p1.y, B0 = p3.x - p1.x, B1 = p3.y - p1.y;
      const double vol = fabs(A0 * B1 - A1 * B0) / 2;
      xc = sqrt(vol);
    }
    c = sum / xc / ntracers;
    mt = sum / xc / (double)cet.enc[e];
  }
  out[e] = c;
  out[m.nelem + e] = mt;
}

void cet_results(const DevMesh& m, const CetDev& cet, int ntracers, double* out, cudaStream_t s) {
  if (m.nelem <= 0) return;
  if (m.dims == 3) k_cet_results<3><<<vblk(m.nelem, 256), 256, 0, s>>>(m, cet, (double)ntracers, out);
  else k_cet_results<2><<<vblk(m.nelem, 256), 256, 0, s>>>(m, cet, (double)ntracers, out);
}

// OutputRT, ompVC/residencetime.c:160-178: -1 for tracers that never were
// in the domain (LeftDomainTime = -1), else the time from the release to
// leaving the domain, or to the release's stop time for tracers still in it.
__global__ void k_residence(TracerDev t, double launch, double stop, double* rt) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= t.n) return;
  const double ldt = t.ldt[i];
  rt[i] = fabs(ldt + 1) < FVC_TINY ? -1.0 : (t.left[i] ? ldt : stop) - launch;
}

void tracer_residence(const TracerDev& t, double launch, double stop, double* rt, cudaStream_t s) {
  if (t.n > 0) k_residence<<<vblk(t.n, 256), 256, 0, s>>>(t, launch, stop, rt);
}

}  // namespace fvc
