// swe_layout.cuh -- the order in which an instance's cells, edges and nodes
// are stored on the device (host code).
//
// Every cell is computed from its own topology row (its nodes, edges and
// neighbours in the caller's local order k = 0, 1, 2) and every edge from its
// own row (owner first, nodes in the caller's order), so a permutation of the
// cells, edges and nodes changes where values live, never the arithmetic: the
// state after any number of steps is bit-identical in every layout.  The
// boundary (swe_abi.cu) translates each array that crosses it back to the
// caller's numbering (the reference has one layout, the caller's,
// include/TriangMesh.h:14-65).
#pragma once

#include <cstdint>
#include <vector>

#include "swe_engine.cuh"

namespace swe {

// Cell orders (device position -> caller's cell).
// Morton: z-order of the centroids on a 2^21 x 2^21 grid over the bounding box.
std::vector<int64_t> morton_cells(const HostInstance& h);
// Reverse Cuthill-McKee over the cell-neighbour graph, one connected
// component after another, each started from a pseudo-peripheral cell.
std::vector<int64_t> rcm_cells(const HostInstance& h);

// The whole layout for a cell order: edges follow their owner cell (in its
// local edge order), nodes their first cell; edges and nodes that no cell
// lists keep their relative order at the end.
Layout layout_from_cells(const HostInstance& h, int strategy, std::vector<int64_t>&& cell_from);
Layout make_layout(const HostInstance& h, int strategy);

// Rewrites h in the device order of L (indices renumbered, rows moved).
HostInstance apply_layout(const HostInstance& h, const Layout& L);

// Cost model of a layout: distinct 32-byte sectors that warps of 32
// consecutive threads touch in the indirect (gathered) reads of the step's
// kernels, summed over warps and weighted by the FP64 arrays read through each
// index (cell kernels: 4 arrays through the neighbours, 2 through the nodes,
// 3 through the edges; edge kernel: 3 arrays through the (slot, cell) pairs of
// owner and neighbour).  Coalesced reads of a thread's own row are the same
// in every layout and not counted.
double gather_sectors(const HostInstance& h_in_device_order);

// kLayoutAuto: the candidate (keep, Morton, RCM) with the fewest sectors;
// the caller's order is kept unless another one saves more than 5 %.
// cost3 (optional) receives the three candidates' costs; applied (optional)
// receives h rewritten in the chosen order.
Layout choose_layout(const HostInstance& h, int strategy, double* cost3, HostInstance* applied);

}  // namespace swe
