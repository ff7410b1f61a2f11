// Tile layout of the FP32 engine: a mesh cut into tiles of up to kTileCore Hilbert-consecutive cells,
// each tile carrying everything one RK stage of its cells needs in a few contiguous blocks, so that a
// stage is ONE kernel: per tile it bulk-copies (TMA) the tile's blocks into shared memory, gathers
// the states of its halo cells, computes the limited gradients of its core cells and of their
// neighbours (ring 1; their gradients need the states of ring 2), the fluxes of every face of its
// core cells, and the residual and RK update of its core cells.  No face value or gradient goes
// through device memory between the gradient, flux and update passes.
//
// Per tile (all ids solve-local; the device adds the solve's base offsets):
//   cells   local slots [0, ncore) core cells (device order c0 .. c0+ncore-1),
//           [ncore, ncore+n1) ring 1, [ncore+n1, ncore+n1+n2) ring 2; halo[] lists ring 1 then ring 2
//   records one per face the tile needs: [0, nrc) every face of a core cell (fluxes are computed for
//           these; the first ncc join two core cells, the first nint join two cells, the rest are
//           boundary faces), [nrc, ngeo) boundary faces of ring-1 cells,
//           [ngeo, nr) the other faces of ring-1 cells (gradient only).  Record block, 4-byte words:
//             sl[nrp]   (s1 & 0xFFFF) | (s2 << 16): local slots of the face's c1 and c2 (s2 < 0: BC code)
//             d[nrp][4] (d1x, d1y, d2x, d2y): face centre minus c1 / c2 centre (c2: ghost centre for
//                       boundary faces), so the LSQ displacement is d1 - d2; one 16-byte row per
//                       record, read (and, by the flux pass, overwritten) with one 128-bit access
//             nx[ngp] ny[ngp] A[ngp]                normal and area of records [0, ngeo)
//           nrp = nr and ngp = ngeo rounded up to 4 (16-byte rows)
//   csr     u16 words: off[noff] (ngrad+1 entry offsets, padded to 8 words; bit 15 of a cell's end
//           offset off[g+1] is set when the cell has a boundary face) then 32-bit entries of
//           every core and ring-1 cell, each cell's in ascending ORIGINAL face id (the reference's
//           summation order), padded to 4 entries: low half (record << 1 | side), high half the local
//           slot of the face's other cell (or its BC code, < 0) as int16, so the gradient pass needs
//           no lookup of the record's slots
//   qcell   per record: NO_SLIP_WALL gradient ghost cell (the cell numbered like the face's original
//           id, src/solver/cell_gradient.cpp:63-66), -1 otherwise
#pragma once

#include <array>
#include <cstdint>
#include <string>
#include <vector>

namespace fv2d {

constexpr int kTileCore = 256;     // core cells per tile at most (threads per CTA)
constexpr int kTileGrad = 400;     // core + ring-1 cells at most
constexpr int kTileCells = 560;    // core + ring-1 + ring-2 cells at most
constexpr int kTileRecs = 1344;    // records at most
constexpr int kTileGeo = 960;      // records with normal and area at most
constexpr int kTileCsr = 5528;     // u16 words of the csr block at most (offsets + 32-bit entries)
// (the largest tiles of a 1M-cell Voronoi mesh: 382 gradient cells, 518 cells, 1,272 records, 889
// with geometry, 2,300 csr entries; a block over a capacity is halved)

// One tile, solve-local offsets.
struct TileRec {
    long long rec = 0;     // word offset of the record block
    long long rbase = 0;   // index of the tile's first record (qcell)
    long long csr = 0;     // u16 offset of the csr block
    long long halo = 0;    // int offset of the halo list
    int c0 = 0, ncore = 0, n1 = 0, n2 = 0;
    int ncc = 0, nint = 0, nrc = 0, ngeo = 0, nr = 0, nrp = 0, ngp = 0;
    int noff = 0, ncsr = 0;        // u16 words: offsets part, whole block (both multiples of 8)
    int nhalo = 0;                 // ints of the halo list (n1 + n2 rounded up to 4)
};

// Device descriptor of one tile: the solve-local TileRec plus the arena bases of its solve.
struct TileDesc {
    long long rec, rbase, csr, halo;
    int cbase;             // arena id of the solve's cell 0 (halo ids and qcell are solve-local)
    int c0;                // arena id of the tile's first core cell
    int ncore, n1, n2;
    int nrc, ngeo, nr, nrp, ngp;
    int noff, ncsr, nhalo;
    int sid;
    int ncc;               // flux records joining two core cells (the first ncc)
    int fpw;               // flux records a warp takes per grab (a multiple of 32; the batch's tuning)
    int nint;              // flux records joining two cells (the first nint; ncc <= nint <= nrc)
    int pad0, pad1, pad2;
};
static_assert(sizeof(TileDesc) == 112, "TileDesc layout");

struct TileLayout {
    int nc = 0;                          // cells (device order)
    int nc4 = 0;                         // cells rounded up to 4 (per-cell arrays are this long)
    std::vector<TileRec> tiles;
    std::vector<uint32_t> rec;           // record blocks
    std::vector<int> qcell;              // per record
    std::vector<uint16_t> csr;           // csr blocks
    std::vector<int> halo;               // halo lists
    // per cell, device order, nc4 entries: volume and its reciprocal; the LSQ inverse-moment terms
    // (Ixx, Iyy, Ixy, 0) rounded from FP64 to FP32 (the kernels' gradient reads one 16-byte row)
    std::vector<float> vol, rvol;
    std::vector<std::array<float, 4>> lsq;
    // statistics: records per face, ring-1 and ring-2 cells per cell
    double rec_per_face = 0, ring1_per_cell = 0, ring2_per_cell = 0;
};

struct HostMesh;
struct DeviceLayout;
// Build the tile layout of a mesh (device order from build_layout).  Returns false (with a
// message) only if a single cell needs more than a tile's capacity.
bool build_tile_layout(const HostMesh& m, const DeviceLayout& L, TileLayout& T, std::string& err);
// Every index the stage kernels derive from the layout stays inside its array or shared-memory
// region (run by build_tile_layout before a layout is used).
bool check_tile_layout(const TileLayout& T, const DeviceLayout& L, std::string& err);

}  // namespace fv2d
