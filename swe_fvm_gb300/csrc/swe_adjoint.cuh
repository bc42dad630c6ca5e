// swe_adjoint.cuh -- work arrays of the discrete adjoint (see swe_adjoint.cu).
#pragma once

#include "swe_engine.cuh"

namespace swe {

// Forward-only part of a partially-wet cell's reconstruction reverse.
struct PwJac {
  double w0, gx, gy;  // the forward plane (level, slope)
  // plane: d(w0, gx, gy) / d(w, w23, z_lo, z_mid, z_hi); PartWet1 level:
  // jw0[0..3] = d level / d(w, z0, z1, z2)
  double jw0[5], jgx[5], jgy[5];
  // where w23 (the PartWet2 node maximum) came from: route 0 node `target`;
  // 1 dry cell `target` (rc[0..2] to its nodes); 2 fully-wet cell `target`
  // (its level; rc[0..2] plane-point weights of combination `mask` when
  // mask >= 0); 3 PartWet1 cell `target` (rc[0] its level, rc[1..3] its nodes)
  double rc[4];
  int plane, route, target, mask;
};

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
  PwJac* pwjac;                               // [C] partially-wet cells' Jacobians
  // [C][8][6] adjoint of the fully-wet combination plane's point z: for
  // neighbour mask q, lp_k = lg0 padj[.][q][k] + lg1 padj[.][q][3 + k]
  // (geometry only; zero for cells next to a wall, which are never fully wet)
  double* padj;
  // depth below which the w-slope of a PartWet1 level feeding a node maximum
  // is regularised (the reference's kEta1 = 1e-3 by default; 0: the exact
  // derivative of the discrete forward)
  double reg_depth;
};

}  // namespace swe
