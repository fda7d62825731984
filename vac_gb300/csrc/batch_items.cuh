// batch_items.cuh - the work list of a batch of grids: what a persistent
// sweep kernel reads per work item (batch.cu builds the lists; the fused
// and pair sweep units hold the kernels that walk them).
#pragma once
#include "control.cuh"
#include "sweep_fused.cuh"

namespace vacgpu {

// one work item: a tile (bx, by) and z chunk bz of grid inst (2-D line
// sweeps: strip bx with the sweep direction in bit 30, rows by .. bz-1)
struct BItem {
  int inst, bx, by, bz;
};

// one grid of the batch
struct BInst {
  FusedArgs fa;        // wout chosen per sweep from buf[] and Ctrl::cur
  SweepArgs sa;        // first-step passes
  float* buf[2];
};

// The launch of the pair sweep over a batch work list (sweep_pair.cu):
// `ctas` persistent CTAs (0: one per item) walk items[0..nitems); sweep:
// index of the sweep within the step (its parity picks the source buffer);
// gen: the general form (some grid has pair_general).  False if the pair
// kernel has no instance for (D, mhd, lim).
bool launch_batch_pair(const BItem* items, int nitems, const BInst* insts,
                       const CUtensorMap* maps, int sweep, int D, bool mhd, int lim,
                       bool gen, int ctas, cudaStream_t st);

// The grid needs the general form of the pair sweep: gravity, a
// non-periodic face, split sources, no Powell terms for MHD, or no CFL
// maximum.
bool pair_general(const FusedArgs& a, bool mhd);

// The pair sweep applies to a grid (3-D, one limiter for every variable,
// minmod or woodward, even row offsets); also false when VACGPU_PAIR=0.
bool pair_applies(const FusedArgs& a, bool mhd);

// Strips of the 2-D line sweep along D over nx mesh columns: 60 output
// columns a strip (64 for the HD y sweep, which needs no halo columns).
__host__ __device__ inline int line2_strips(int D, bool mhd, int nx) {
  const int tw = (D == 0 || mhd) ? 60 : 64;
  return (nx + tw - 1) / tw;
}

// State of the grid-wide barrier of a cooperative launch, in device
// memory: arrivals, generation (advanced by the last arrival), a fault flag
// (a barrier wait gave up), per step parity whether some grid needs the
// first-step passes, and the next unclaimed work item of the first and the
// second sweep of a step.
struct GridSync {
  unsigned count, gen;
  int fault;
  int need[2];
  int next[2];
};

// Every step of a 2-D line-sweep batch in one cooperative launch
// (sweep_line2.cu): per step the control of each grid (dt choice), the
// first-step passes where a grid needs them, both sweeps over their work
// lists and the step epilogue, separated by grid-wide barriers.
struct Line2Steps {
  const BItem* items[2];  // work lists of the x and y sweeps
  int nitems[2];
  const BInst* insts;
  Ctrl* const* ctrls;
  int n;                  // grids
  int nsteps;             // steps at most (each grid stops as VAC would)
  double tstop;
  int par0;               // parity of it at the first step
  int xy;                 // typedimsplit 'xy' (else 'xyyx')
  DtEndArgs dte;
  double smallpcoeff;
  int nparts;             // blocks per grid of the first-step passes
  GridSync* gs;
};

// Resident CTAs of the cooperative kernel for (mhd, lim, gen) on this
// device, and its launch (false: no instance, or the launch was refused).
int line2_steps_ctas(bool mhd, int lim, bool gen);
bool launch_line2_steps(const Line2Steps& ls, bool mhd, int lim, bool gen, int ctas,
                        cudaStream_t st);

// The same for 2-D grids and the warp-marching sweep (sweep_line2.cu),
// whose work items are (grid, strip bx, output rows by .. bz-1 as
// ghost-range indices) and whose launch runs `ctas` CTAs of four warps (0:
// one warp per item).
bool line2_applies(const FusedArgs& a, bool mhd);
bool launch_batch_line2(const BItem* items, int nitems, const BInst* insts, int sweep, int D,
                        bool mhd, int lim, bool gen, int ctas, cudaStream_t st);

}  // namespace vacgpu
