// swe_adjoint.cuh -- work arrays of the discrete adjoint (see swe_adjoint.cu).
#pragma once

#include "swe_engine.cuh"

namespace swe {

struct AdjWork {
  double* lam;   // [3][C] adjoint of the stage output (w, u, v)
  double* lamp;  // [3][C] adjoint of the stage input, accumulated
  double* lam0;  // [3][C] adjoint of the step's initial state through the Shu-Osher terms
  double *lew, *leu, *lev, *lsx, *lsy, *lze;  // [3C] per interface slot
  double *lF0, *lF1, *lF2;                    // [3C] per slot: the cell's share of the edge-flux adjoint
  double* lF0d;                               // [3C] per slot: draining-time-step share of dF0
  double* ldtk;                               // [3C] adjoint of the slot's selected draining time step
  unsigned char* route;                       // [3C] 0 none, 1 own draining dt, 2 the neighbour's
  double* lhwall;                             // [3C] wall-flux depth adjoint (owner slot)
  double* lbc;                                // [C] centroid-bathymetry adjoint
  double* lscatter;                           // [C] node-maximum scatter into other cells
  double* lz;                                 // [N] node-bathymetry gradient
  const int* twin;                            // [3C] slot of the neighbour on the same edge, -1 at walls
  const int* node_ptr;                        // [N+1] cells around each node (CSR)
  const int* node_cells;                      // (cell << 2) | local node index
  const int* edge_nodes;                      // [2E] global node ids of each edge
};

}  // namespace swe
