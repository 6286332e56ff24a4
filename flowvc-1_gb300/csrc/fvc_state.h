// fvc_state.h -- plain-old-data views of the device-resident mesh, velocity
// window and integrator settings, passed by value to every kernel.
#pragma once
#include <cuda_runtime.h>

namespace fvc {

// per-point fault bits, OR-ed into a launch's status word
enum : int { PT_ERR_WALK = 1, PT_ERR_TLOC = 2, PT_ERR_STATE = 4, PT_ERR_CET = 8 };
// the element id a neighbour walk leaves behind when it fails (the hop cap,
// or ompVC's "Indeterminate neighbor"); a boundary exit leaves -1.  The walk
// stops either way, and the fault becomes PT_ERR_WALK where the callers
// handle a point's stop, outside the stepping loop.
enum : int { EID_FAULT = -2 };

struct DevMesh {
  int dims, mesh_type;  // 2/3; 0 Cartesian, 1 unstructured
  // Cartesian velocity grid (Vel_CartMesh, ompVC/mesh.c:67-122)
  double xmin, ymin, zmin, dx, dy, dz;
  double rdx, rdy, rdz;  // reciprocals for div_rn (0: divide)
  int xres, yres, zres;
  // unstructured mesh
  const int4* elem;     // 2 x nelem: {Nodes[4]}, {NeighborIndex[4]}
  const double* geom;   // natural-coordinate map + node ids, 16 (3D) or 12 (2D) doubles per element
  const float* geo32;   // FP32 copy of the map, node-0 coordinates and error scale, 64 B per element
  const float4* geo32lo;  // node 0's coordinates minus their FP32 copies in geo32 (x, y, z, 0)
  const double4_32a* nodes; // x, y, z, 0 per node
  int nelem, nnodes;
  // Data_MeshBounds
  double bounds[6];
  int max_hops;
  int prec;  // arithmetic form: FVC_PREC_FP64 (ompVC's, bit-exact) or a mixed form
};

// One step of a call's step sequence for the mixed-precision form: the
// step's start time (exact, as the FP64 host loop computes it), its length
// and the tloc of its three stage times.  Entry nsteps holds the end time.
struct StepM {
  double tc;
  float h;
  float tl0, tlh, tl1;
  float pad[3];
};

// Stage times of one advection call.  Every particle of a call starts at the
// same t1 with the same step h, so the reference's stage times
// tc_k, tc_k + h_k/2 and tc_k + h_k (= tc_{k+1}) form one table; slot 2k is
// tc_k, slot 2k+1 is tc_k + h_k/2.
#define FVC_MAX_SLOTS 40

// Two resident frames bracketing [tmin, tmax] (Data_LoadedTMin/TMax), and
// the stage-time table of the current call.  For unstructured meshes vt holds
// the frames interpolated to every slot's time at every node, computed once
// per call with the reference's expression (1 - tloc)*U0 + tloc*U1, so a
// stage evaluation reads the same doubles it would compute.
struct DevWindow {
  const double4_32a* f0;  // frame at tmin, (u, v, w, 0) per node
  const double4_32a* f1;  // frame at tmax
  double tmin, tmax;
  double rspan;           // reciprocal of tmax - tmin for div_rn (0: divide)
  const double4_32a* vt;  // nslots x vt_stride time-interpolated node velocities
  long vt_stride;
  int nslots;
  double tq[FVC_MAX_SLOTS];  // slot times
  double tl[FVC_MAX_SLOTS];  // tloc of each slot, range-checked when the table is built
  // mixed-precision form: the two frames quantised to 16 bits a component
  // with a per-frame, per-component FP32 scale, interleaved per node in one
  // 16-byte record (u0 v0 | w0 u1 | v1 w1 | -) so a stage reads one sector a
  // node; and the call's step table
  const uint4* qp;
  float qs0[3], qs1[3];
  int qfmt;  // FVC_PREC_BF16 or FVC_PREC_FP16
  const StepM* steps;
  int nsteps;
  // Cartesian 2D: both frames' w components are all +0.0, so the w sum of
  // GetVelocity_Cartesian is +0.0 and is not computed
  int wz;
};

// Uniform bucket grid over the mesh for Get_Element_Global_Search.
struct BucketGrid {
  double lo[3], inv[3];   // origin and 1 / cell size
  int n[3];               // cells per axis
  const int* start;       // ncells + 1 offsets
  const int* ids;         // element ids per cell, ascending
};

// Exposure-time accumulators (Trace_CETArray, ompVC/exposuretime.c:110-172):
// per element of the velocity mesh, the time tracers spent in it and the
// number of times one entered it.  Shared by every release of a run.
struct CetDev {
  double* sum;   // CETsum
  int* enc;      // Encounters
  int substeps;  // Trace_CETSubsteps (>= 2)
  BucketGrid g;  // global-search fallback of the sub-step walk
};

// Where an integrator writes the position after each accepted step: after
// its k-th accepted step (k = 1 .. max) at base + (k - 1) stride (FP64 form:
// 3 doubles; mixed form: 3 (X, c) float pairs).
struct RecOut {
  double* base;
  long stride;
  int max;
  // RK4: the element state after step 1 (stage hints 1-3 and the located
  // element), when stage 1 stayed in the start element eid0 (else x = -3)
  int4* e1;
  int eid0;
};

// An early-FTLE advection that started from another element hint than the
// main pass: after its step 1 it stops (hit = 1) if its element state is the
// main pass's (stage hints e0 and e1.xyz, located element e1.w), from where
// the rest of its steps are the main pass's record.
struct Chk1 {
  int e0;
  int4 e1;
  int hit;
};

struct DevInteg {
  int type;  // 0 Euler, 1 RK4, 2 RKF, 3 AB2
  double h;  // Int_TimeStep
  int extrapolate;
  double acc, hmin, hmax;  // Int_Accuracy, Int_MinTimeStep, Int_MaxTimeStep (RKF)
};

}  // namespace fvc
