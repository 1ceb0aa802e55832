// Host-side unstructured 2-D mesh: topology, geometry, cell ordering,
// colouring and synthetic generators for the steady-flow hot path.
//
// Semantics follow the reference's UMesh (src/mesh/mesh.hpp, mesh.cpp):
//  * cells are linear triangles/quads with counter-clockwise nodes;
//  * local edge j of a cell joins its nodes j and (j+1) mod nnode;
//  * faces: physical-boundary faces first (in input order), then interior
//    faces ordered by (lower cell, local edge of the lower cell), with the
//    lower-index cell on the left; unit normals point left -> right and,
//    on boundary faces, out of the domain (mesh.cpp:660-763, 347-366).
// The build is independent of the reference's algorithm: edges are matched
// by sorting node-pair keys instead of elements-surrounding-points sweeps.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace fvg {

struct HostMesh {
	int npoin = 0, nelem = 0, nbface = 0, ninface = 0, naface = 0;
	std::vector<double> coords;   // npoin x 2
	std::vector<int> nnode;       // nelem (3 or 4)
	std::vector<int> inpoel;      // nelem x 4, -1 padded
	std::vector<int> bface;       // nbface x 2 nodes, oriented with the host cell
	std::vector<int> btag;        // nbface
	std::vector<int> perm;        // new cell k = input cell perm[k]

	// topology
	std::vector<int> face_l, face_r;      // naface; boundary faces: face_r = -1 - ib
	std::vector<int> face_n0, face_n1;    // naface nodes
	std::vector<int> face_sl, face_sr;    // local edge index of the face in its left/right cell
	std::vector<int> esuel;               // nelem x 4: neighbour cell, -1-ib for boundary, INT_MIN unused
	std::vector<int> elemface;            // nelem x 4
	// geometry
	std::vector<double> area;             // nelem
	std::vector<double> cc;               // nelem x 2 (node averages)
	std::vector<double> fnorm;            // naface x 3 (nx, ny, len)
	std::vector<double> fc;               // naface x 2 (face centre)
	std::vector<double> gc;               // nbface x 2 ghost-cell centres (mid-point reflection)
	// multicolour ordering of the cell adjacency graph (interior faces)
	int ncolors = 0;
	std::vector<int> color;               // nelem
	std::vector<int> color_ptr, color_cells;
	// lines of strongly coupled cells (find_lines); empty unless requested
	std::vector<std::vector<int>> lines;
	std::vector<int> cell_line;           // nelem: line of the cell or -1

	int build(std::string *err);          // topology + geometry + colouring
	int check(std::string *err) const;    // positive areas, closed cells
};

/* Creates a mesh from raw arrays.  reorder: 0 keep input order, 1 reverse
 * Cuthill-McKee.  Cells with clockwise nodes are flipped. */
int mesh_from_arrays(HostMesh &m, int npoin, const double *coords, int nelem, const int *nnode, const int *inpoel,
                     int nbface, const int *bface, const int *btag, int reorder, std::string *err);

/* Block-colour elimination order for the SGS / ILU(0) preconditioners:
 * cells are split into parts of at most part_size cells grown breadth-first
 * over the cell graph (each from the lowest-numbered free cell), parts sharing a face get different
 * colours (when the mesh has lines, find_lines, a part takes whole lines --
 * lines longer than a part in consecutive pieces -- so that the strong
 * couplings along a line are eliminated inside one part), and the order is
 * colour-major, then part-major, then inside a part
 * by dependency level (ties by cell index).  Within a part the relative order
 * of any two adjacent cells is their index order, so ILU(0) on this order
 * equals ILU(0) on the cell order with the couplings between same-colour parts
 * absent (there are none); the levels let one CTA sweep a part with a barrier
 * between levels. */
struct BlockOrder {
	int nparts = 0, ncolors = 0, max_width = 0;
	std::vector<int> pos_cell;   // elimination position -> cell
	std::vector<int> part_ptr;   // part -> position range
	std::vector<int> cpart_ptr;  // colour -> part range
	std::vector<int> lev_ptr;    // part -> range in lev_pos
	std::vector<int> lev_pos;    // level start positions (each part's levels in order)
};
/* colouring: 0 greedy in part order, 1 DSatur with Kempe-chain interchanges
 * (usually one colour fewer) */
BlockOrder block_colour_order(const HostMesh &h, int part_size, int colouring = 0);

/* Lines of strongly coupled cells (findLines / computeWeights,
 * meshordering.cpp:131-262): the weight of a cell's interior neighbour is
 * (1/centroid distance) over the smallest such value about the cell; from the
 * cell of each physical boundary face (in boundary-face order) a line follows
 * the strongest-weighted neighbour not yet in a line while that weight exceeds
 * threshold; lines of one cell are dropped.  Stores h.lines, h.cell_line and
 * returns the number of lines. */
int find_lines(HostMesh &h, double threshold);

/* Periodic pairing of the boundary faces of marker bcm (UMesh::compute_periodic_map,
 * mesh.cpp:368-421): two faces pair when their centres' coordinate along the
 * axis other than `axis` agrees to 1e-8, the first unpaired later face
 * winning.  map[f] = partner face (boundary-face index) or -1. */
std::vector<int> periodic_map(const HostMesh &h, int bcm, int axis);

/* Reverse Cuthill-McKee ordering of the cell graph (own implementation:
 * George-Liu pseudo-peripheral start, neighbours visited by increasing degree). */
std::vector<int> rcm_order(int n, const std::vector<int> &adj_ptr, const std::vector<int> &adj);

// ---- synthetic meshes (seeded, deterministic integer choices) ----

/* Gaussian-bump channel: x in [-1.5,1.5], y in [yb(x), 0.8], yb = 0.0625 exp(-25 x^2);
 * nx x ny quads with exactly round(split_frac*nx*ny) of them (seeded) split
 * into two triangles along a seeded diagonal.
 * Markers: 1 bottom wall, 2 outlet (x=1.5), 3 top wall, 4 inlet (x=-1.5). */
struct RawMesh {
	int npoin = 0, nelem = 0, nbface = 0;
	std::vector<double> coords;
	std::vector<int> nnode, inpoel, bface, btag;
};
RawMesh gen_channel_bump(int nx, int ny, double split_frac, uint64_t seed);

/* NACA 0012 (closed trailing edge) O-grid: nc points around the airfoil
 * (cosine clustering), nr rings out to a circle of radius rfar about
 * (0.5,0).  Ring distances: nbl geometric rings with first height h0 and
 * growth gbl, then (nr - nbl) geometric rings whose growth is solved so the
 * last ring reaches the far field.  Rings with index >= tri_from are split into
 * triangles along seeded diagonals.  Markers: 2 airfoil wall, 4 far field. */
RawMesh gen_naca_ogrid(int nc, int nr, double rfar, int nbl, double h0, double gbl, int tri_from, uint64_t seed);
RawMesh gen_naca_hybrid(int nc, int nbl, double h0, double gbl, double rfar, double beta);

/* Gmsh 2.2 ASCII reader: line elements (type 1) are boundary faces with
 * their first tag as marker; triangles (2) and quads (3) are cells. */
int read_gmsh2(const std::string &path, RawMesh &out, std::string *err);

/* SU2 ASCII reader (2-D): NELEM cells (VTK types 5 triangle, 9 quad, 0-based
 * node indices), NPOIN coordinates, NMARK markers with numeric MARKER_TAG whose
 * line elements (type 3) are boundary faces. */
int read_su2(const std::string &path, RawMesh &out, std::string *err);

}  // namespace fvg
