/* ORACLE — test infrastructure only.
 *
 * A CPU (FP64, OpenMP) restatement of the reference's steady implicit hot
 * path, used by the tests as the parity checker and by bench.py as the timed
 * CPU baseline.  The product never links, loads or calls anything in this
 * directory.
 *
 * Restated from (reference paths):
 *   mesh topology / geometry   src/mesh/mesh.cpp:55-80, 291-366, 471-546, 660-763
 *   cell / ghost / face centres src/spatial/aspatial.cpp:36-119
 *   gradients                  src/spatial/agradientschemes.cpp:37-440
 *   reconstructions            src/spatial/areconstruction.cpp:53-103,
 *                              src/spatial/musclreconstruction.cpp:34-130,
 *                              src/spatial/limitedlinearreconstruction.cpp:28-268
 *   residual driver            src/spatial/flow_spatial.cpp:73-93, 348-395, 488-816
 *   Jacobian assembly          src/spatial/aspatial.cpp:242-340, flow_spatial.cpp:818-875
 *   pseudo-time solver         src/ode/aodesolver.cpp:110-120, 300-329, 363-638
 *   nonlinear relaxation       src/ode/nonlinearrelaxation.cpp:25-38
 *   matrix-free J.x            src/linalg/alinalg.cpp:143-237
 *   surface functionals        src/spatial/flow_spatial.cpp:95-112, 130-310
 *   entropy error              src/spatial/aoutput.cpp:28-62
 * Third-party (PETSc, not vendored in the reference; published algorithms):
 *   block ILU(0) / block SOR(SGS) / point-block Jacobi on BAIJ(4), FGMRES(m)
 *   with classical Gram-Schmidt and Givens rotations, zero initial guess,
 *   convergence when ||r_k|| <= rtol ||b||.
 *
 * Deliberate definitions where the reference is undefined (documented in the
 * build's design notes): the Barth-Jespersen and Venkatakrishnan limiters read
 * the neighbour state of a physical-boundary face from the ghost-cell state
 * (the reference indexes past the end of its cell array there), and the
 * limiter parameter is taken from the configuration (the reference never
 * parses it).
 *
 * Face-loop accumulations are done as per-face contributions gathered per
 * cell in ascending face order, so results do not depend on thread count.
 */
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "orc_physics.hpp"

namespace orc {

// =========================== mesh (mesh.cpp) ===============================

struct Mesh {
	int npoin = 0, nelem = 0, nbface = 0, ninface = 0, naface = 0;
	std::vector<double> coords;      // npoin x 2
	std::vector<int> nnode;          // nelem
	std::vector<int> inpoel;         // nelem x 4
	std::vector<int> bface;          // nbface x 2
	std::vector<int> btag;           // nbface
	std::vector<int> esup_p, esup;
	std::vector<int> esuel;          // nelem x 4
	std::vector<int> intfac;         // naface x 4 (left, right, node0, node1)
	std::vector<int> elemface;       // nelem x 4
	std::vector<double> area;        // nelem
	std::vector<double> facemetric;  // naface x 3 (nx, ny, len)
	// cell -> (face, side) lists in ascending face order, for deterministic gathers
	std::vector<int> cf_ptr, cf_face, cf_side;

	double x(int p) const { return coords[2 * p]; }
	double y(int p) const { return coords[2 * p + 1]; }

	/* compute_elementsSurroundingPoints, mesh.cpp:422-468 */
	void compute_esup()
	{
		esup_p.assign(npoin + 1, 0);
		for (int i = 0; i < nelem; i++)
			for (int j = 0; j < nnode[i]; j++) esup_p[inpoel[4 * i + j] + 1]++;
		for (int i = 1; i <= npoin; i++) esup_p[i] += esup_p[i - 1];
		esup.assign(esup_p[npoin], 0);
		std::vector<int> fill(esup_p.begin(), esup_p.end() - 1);
		for (int i = 0; i < nelem; i++)
			for (int j = 0; j < nnode[i]; j++) esup[fill[inpoel[4 * i + j]]++] = i;
	}

	/* getFaceEIndex for a physical boundary face: local edge of lelem whose
	 * two nodes are the bface nodes (mesh.cpp:552-600). */
	int bface_eindex(int iface, int lelem) const
	{
		for (int j = 0; j < nnode[lelem]; j++) {
			const int a = inpoel[4 * lelem + j], b = inpoel[4 * lelem + (j + 1) % nnode[lelem]];
			const int p = bface[2 * iface], q = bface[2 * iface + 1];
			if ((a == p && b == q) || (a == q && b == p)) return j;
		}
		return -1;
	}

	/* compute_phyBFaceNeighboringElements, mesh.cpp:602-656 */
	int bface_host(int iface) const
	{
		const int p = bface[2 * iface], q = bface[2 * iface + 1];
		std::vector<int> a(esup.begin() + esup_p[p], esup.begin() + esup_p[p + 1]);
		std::vector<int> b(esup.begin() + esup_p[q], esup.begin() + esup_p[q + 1]);
		std::sort(a.begin(), a.end());
		std::sort(b.begin(), b.end());
		std::vector<int> c;
		std::set_intersection(a.begin(), a.end(), b.begin(), b.end(), std::back_inserter(c));
		if (c.size() != 1) return -1;
		return c[0];
	}

	/* correctBoundaryFaceOrientation, mesh.cpp:55-80 */
	int correct_bface_orientation()
	{
		for (int f = 0; f < nbface; f++) {
			const int h = bface_host(f);
			if (h < 0) return 1;
			const int e = bface_eindex(f, h);
			if (e < 0) return 1;
			bface[2 * f] = inpoel[4 * h + e];
			bface[2 * f + 1] = inpoel[4 * h + (e + 1) % nnode[h]];
		}
		return 0;
	}

	/* compute_elementsSurroundingElements, mesh.cpp:471-546 */
	void compute_esuel()
	{
		esuel.assign(4 * nelem, -1);
		std::vector<int> lpoin(npoin, 0);
		for (int ie = 0; ie < nelem; ie++) {
			for (int ifa = 0; ifa < nnode[ie]; ifa++) {
				const int h0 = inpoel[4 * ie + ifa], h1 = inpoel[4 * ie + (ifa + 1) % nnode[ie]];
				lpoin[h0] = 1; lpoin[h1] = 1;
				for (int is = esup_p[h0]; is < esup_p[h0 + 1]; is++) {
					const int je = esup[is];
					if (je == ie) continue;
					for (int jfa = 0; jfa < nnode[je]; jfa++) {
						int icoun = 0;
						for (int jn = 0; jn < 2; jn++)
							if (lpoin[inpoel[4 * je + (jfa + jn) % nnode[je]]] == 1) icoun++;
						if (icoun == 2) {
							esuel[4 * ie + ifa] = je;
							esuel[4 * je + jfa] = ie;
						}
					}
				}
				lpoin[h0] = 0; lpoin[h1] = 0;
			}
		}
	}

	/* compute_faceConnectivity, mesh.cpp:660-763 (no connectivity faces) */
	int compute_faces()
	{
		ninface = 0;
		for (int ie = 0; ie < nelem; ie++)
			for (int in = 0; in < nnode[ie]; in++) {
				const int je = esuel[4 * ie + in];
				if (je > ie && je < nelem) ninface++;
			}
		naface = ninface + nbface;
		intfac.assign(4 * naface, -1);
		elemface.assign(4 * nelem, -1);
		for (int f = 0; f < nbface; f++) {
			const int h = bface_host(f);
			const int e = bface_eindex(f, h);
			if (h < 0 || e < 0) return 1;
			intfac[4 * f] = h;
			intfac[4 * f + 1] = nelem + f;
			intfac[4 * f + 2] = bface[2 * f];
			intfac[4 * f + 3] = bface[2 * f + 1];
			esuel[4 * h + e] = nelem + f;
			elemface[4 * h + e] = f;
		}
		int fi = nbface;
		for (int ie = 0; ie < nelem; ie++)
			for (int in = 0; in < nnode[ie]; in++) {
				const int je = esuel[4 * ie + in];
				if (je > ie && je < nelem) {
					const int in1 = (in + 1) % nnode[ie];
					intfac[4 * fi] = ie;
					intfac[4 * fi + 1] = je;
					intfac[4 * fi + 2] = inpoel[4 * ie + in];
					intfac[4 * fi + 3] = inpoel[4 * ie + in1];
					elemface[4 * ie + in] = fi;
					for (int jn = 0; jn < nnode[je]; jn++)
						if (inpoel[4 * ie + in1] == inpoel[4 * je + jn]) elemface[4 * je + jn] = fi;
					fi++;
				}
			}
		return 0;
	}

	/* compute_areas, mesh.cpp:291-314 */
	void compute_areas()
	{
		area.assign(nelem, 0.0);
		auto tri = [&](int a, int b, int c) {
			return 0.5 * (x(a) * (y(b) - y(c)) - y(a) * (x(b) - x(c)) + x(b) * y(c) - x(c) * y(b));
		};
		for (int i = 0; i < nelem; i++) {
			const int *e = &inpoel[4 * i];
			if (nnode[i] == 3)
				area[i] = tri(e[0], e[1], e[2]);
			else {
				area[i] = tri(e[0], e[1], e[2]);
				area[i] += tri(e[0], e[2], e[3]);
			}
		}
	}

	/* compute_face_data, mesh.cpp:347-366 */
	void compute_face_data()
	{
		facemetric.assign(3 * naface, 0.0);
		for (int i = 0; i < naface; i++) {
			const int a = intfac[4 * i + 2], b = intfac[4 * i + 3];
			double nx = y(b) - y(a), ny = -1.0 * (x(b) - x(a));
			const double len = std::sqrt(std::pow(nx, 2) + std::pow(ny, 2));
			facemetric[3 * i] = nx / len;
			facemetric[3 * i + 1] = ny / len;
			facemetric[3 * i + 2] = len;
		}
	}

	void build_cell_face_lists()
	{
		cf_ptr.assign(nelem + 1, 0);
		for (int f = 0; f < naface; f++) {
			cf_ptr[intfac[4 * f] + 1]++;
			if (intfac[4 * f + 1] < nelem) cf_ptr[intfac[4 * f + 1] + 1]++;
		}
		for (int i = 0; i < nelem; i++) cf_ptr[i + 1] += cf_ptr[i];
		cf_face.assign(cf_ptr[nelem], 0);
		cf_side.assign(cf_ptr[nelem], 0);
		std::vector<int> fill(cf_ptr.begin(), cf_ptr.end() - 1);
		for (int f = 0; f < naface; f++) {
			const int l = intfac[4 * f], r = intfac[4 * f + 1];
			cf_face[fill[l]] = f; cf_side[fill[l]++] = 0;
			if (r < nelem) { cf_face[fill[r]] = f; cf_side[fill[r]++] = 1; }
		}
	}

	int build()
	{
		compute_esup();
		if (correct_bface_orientation()) return 1;
		compute_esuel();
		if (compute_faces()) return 2;
		compute_areas();
		compute_face_data();
		build_cell_face_lists();
		return 0;
	}
};

// ====================== spatial discretisation ==============================

enum { G_NONE = 0, G_GREENGAUSS = 1, G_LEASTSQUARES = 2 };
enum { R_NONE = 0, R_VANALBADA = 1, R_BARTHJESPERSEN = 2, R_VENKATAKRISHNAN = 3, R_WENO = 4 };

struct Disc {
	const Mesh *m = nullptr;
	Phys P;
	double aoa = 0;
	bool viscous = false, constvisc = false;
	int flux = F_ROE, fluxjac = F_ROE, gradscheme = G_LEASTSQUARES, recon = R_NONE;
	double limparam = 0;
	bool order2 = true;
	std::map<int, BCSpec> bcs;
	double uinf[4];
	std::vector<double> rc, rcbp, gr;  // cell centres, ghost centres, face centres
	std::vector<double> Vinv;          // WLS 2x2 inverses (row-major) per cell
	std::vector<double> clength;       // Venkatakrishnan length scale

	int nelem() const { return m->nelem; }

	/* Spatial ctor, aspatial.cpp:36-76, 97-119; WLS ctor agradientschemes.cpp:219-317;
	 * Venkatakrishnan ctor limitedlinearreconstruction.cpp:180-205 */
	int setup()
	{
		const Mesh &M = *m;
		freestream_state(P, aoa, uinf);
		rc.assign(2 * M.nelem, 0.0);
		for (int i = 0; i < M.nelem; i++)
			for (int d = 0; d < 2; d++) {
				double s = 0;
				for (int j = 0; j < M.nnode[i]; j++) s += M.coords[2 * M.inpoel[4 * i + j] + d];
				rc[2 * i + d] = s / (double)M.nnode[i];
			}
		gr.assign(2 * M.naface, 0.0);
		for (int f = 0; f < M.naface; f++) {
			for (int v = 0; v < 2; v++)
				for (int d = 0; d < 2; d++) gr[2 * f + d] += M.coords[2 * M.intfac[4 * f + 2 + v] + d];
			for (int d = 0; d < 2; d++) gr[2 * f + d] /= 2;
		}
		rcbp.assign(2 * M.nbface, 0.0);
		for (int f = 0; f < M.nbface; f++) {
			const int ie = M.intfac[4 * f];
			for (int d = 0; d < 2; d++) {
				double mid = 0;
				for (int v = 0; v < 2; v++) mid += M.coords[2 * M.intfac[4 * f + 2 + v] + d];
				mid /= 2;
				rcbp[2 * f + d] = 2.0 * mid - rc[2 * ie + d];
			}
		}
		for (int f = 0; f < M.nbface; f++)
			if (!bcs.count(M.btag[f])) return 3;
		if (gradscheme == G_LEASTSQUARES) {
			std::vector<double> V(4 * M.nelem, 0.0);
			auto add = [&](int ie, double w2, const double *dr) {
				for (int i = 0; i < 2; i++)
					for (int j = 0; j < 2; j++) V[4 * ie + 2 * i + j] += w2 * dr[i] * dr[j];
			};
			for (int f = 0; f < M.nbface; f++) {
				const int ie = M.intfac[4 * f];
				double w2 = 0, dr[2];
				for (int d = 0; d < 2; d++) {
					w2 += (rc[2 * ie + d] - rcbp[2 * f + d]) * (rc[2 * ie + d] - rcbp[2 * f + d]);
					dr[d] = rc[2 * ie + d] - rcbp[2 * f + d];
				}
				add(ie, 1.0 / w2, dr);
			}
			for (int f = M.nbface; f < M.naface; f++) {
				const int ie = M.intfac[4 * f], je = M.intfac[4 * f + 1];
				double w2 = 0, dr[2];
				for (int d = 0; d < 2; d++) {
					w2 += (rc[2 * ie + d] - rc[2 * je + d]) * (rc[2 * ie + d] - rc[2 * je + d]);
					dr[d] = rc[2 * ie + d] - rc[2 * je + d];
				}
				add(ie, 1.0 / w2, dr);
				add(je, 1.0 / w2, dr);
			}
			Vinv.assign(4 * M.nelem, 0.0);
			for (int i = 0; i < M.nelem; i++) {
				const double a = V[4 * i], b = V[4 * i + 1], c = V[4 * i + 2], d = V[4 * i + 3];
				const double det = a * d - b * c;
				Vinv[4 * i] = d / det; Vinv[4 * i + 1] = -b / det;
				Vinv[4 * i + 2] = -c / det; Vinv[4 * i + 3] = a / det;
			}
		}
		if (recon == R_VENKATAKRISHNAN) {
			clength.assign(M.nelem, 0.0);
			for (int i = 0; i < M.nelem; i++) {
				for (int k = 0; k < M.nnode[i]; k++) {
					const int a = M.inpoel[4 * i + k], b = M.inpoel[4 * i + (k + 1) % M.nnode[i]];
					double l = 0;
					for (int d = 0; d < 2; d++) l += std::pow(M.coords[2 * a + d] - M.coords[2 * b + d], 2);
					if (clength[i] < l) clength[i] = l;
				}
				clength[i] = std::sqrt(clength[i]);
			}
		}
		return 0;
	}

	const BCSpec &bc_of_face(int f) const { return bcs.at(m->btag[f]); }

	/* compute_boundary_state, flow_spatial.cpp:85-93 */
	void boundary_state(int f, const double *ins, double *gs) const
	{
		ghost_state(P, bc_of_face(f), uinf, ins, &m->facemetric[3 * f], gs);
	}

	// ---------- gradients (agradientschemes.cpp) ----------
	/* u: nelem x 4 (cell values), ug: nbface x 4 ghost values; grad: nelem x 8
	 * laid out as GradBlock_t (column-major 2 x 4: (x,v0),(y,v0),(x,v1),...). */
	void gradients(const double *u, const double *ug, double *grad) const
	{
		const Mesh &M = *m;
		const int ne = M.nelem, nf = M.naface, nb = M.nbface;
		if (!order2 || gradscheme == G_NONE) {
			std::fill(grad, grad + 8 * ne, 0.0);
			return;
		}
		// per-face contributions to left (c0) and right (c1) cells, 8 values each
		std::vector<double> c0(8 * (size_t)nf), c1(8 * (size_t)nf);
		if (gradscheme == G_GREENGAUSS) {
			/* GreenGaussGradients::compute_gradients, agradientschemes.cpp:62-216 */
#pragma omp parallel for schedule(static)
			for (int f = 0; f < nf; f++) {
				const int ie = M.intfac[4 * f], je = M.intfac[4 * f + 1];
				double mid[2] = {0, 0};
				for (int v = 0; v < 2; v++)
					for (int d = 0; d < 2; d++) mid[d] += M.coords[2 * M.intfac[4 * f + 2 + v] + d];
				for (int d = 0; d < 2; d++) mid[d] /= 2;
				const double *rr = f < nb ? &rcbp[2 * f] : &rc[2 * je];
				const double *uR = f < nb ? &ug[4 * f] : &u[4 * je];
				double dL = 0, dR = 0;
				for (int d = 0; d < 2; d++) {
					dL += (mid[d] - rc[2 * ie + d]) * (mid[d] - rc[2 * ie + d]);
					dR += (mid[d] - rr[d]) * (mid[d] - rr[d]);
				}
				dL = 1.0 / std::sqrt(dL);
				dR = 1.0 / std::sqrt(dR);
				const double ai1 = 1.0 / M.area[ie];
				const double ai2 = f < nb ? 0.0 : 1.0 / M.area[je];
				for (int v = 0; v < 4; v++) {
					const double ut = (u[4 * ie + v] * dL + uR[v] * dR) / (dL + dR) * M.facemetric[3 * f + 2];
					for (int d = 0; d < 2; d++) {
						c0[8 * f + 2 * v + d] = (ut * M.facemetric[3 * f + d]) * ai1;
						c1[8 * f + 2 * v + d] = -((ut * M.facemetric[3 * f + d]) * ai2);
					}
				}
			}
#pragma omp parallel for schedule(static)
			for (int i = 0; i < ne; i++) {
				double g[8] = {0, 0, 0, 0, 0, 0, 0, 0};
				for (int k = M.cf_ptr[i]; k < M.cf_ptr[i + 1]; k++) {
					const double *c = M.cf_side[k] ? &c1[8 * M.cf_face[k]] : &c0[8 * M.cf_face[k]];
					for (int q = 0; q < 8; q++) g[q] += c[q];
				}
				for (int q = 0; q < 8; q++) grad[8 * i + q] = g[q];
			}
		} else {
			/* WeightedLeastSquaresGradients::compute_gradients, agradientschemes.cpp:323-440 */
#pragma omp parallel for schedule(static)
			for (int f = 0; f < nf; f++) {
				const int ie = M.intfac[4 * f], je = M.intfac[4 * f + 1];
				const double *rr = f < nb ? &rcbp[2 * f] : &rc[2 * je];
				const double *uR = f < nb ? &ug[4 * f] : &u[4 * je];
				double w2 = 0, dr[2], du[4];
				for (int d = 0; d < 2; d++) {
					w2 += (rc[2 * ie + d] - rr[d]) * (rc[2 * ie + d] - rr[d]);
					dr[d] = rc[2 * ie + d] - rr[d];
				}
				w2 = 1.0 / w2;
				for (int v = 0; v < 4; v++) du[v] = u[4 * ie + v] - uR[v];
				for (int v = 0; v < 4; v++)
					for (int d = 0; d < 2; d++) {
						c0[8 * f + 2 * v + d] = w2 * dr[d] * du[v];
						c1[8 * f + 2 * v + d] = w2 * dr[d] * du[v];
					}
			}
#pragma omp parallel for schedule(static)
			for (int i = 0; i < ne; i++) {
				double fs[8] = {0, 0, 0, 0, 0, 0, 0, 0};
				for (int k = M.cf_ptr[i]; k < M.cf_ptr[i + 1]; k++) {
					const double *c = M.cf_side[k] ? &c1[8 * M.cf_face[k]] : &c0[8 * M.cf_face[k]];
					for (int q = 0; q < 8; q++) fs[q] += c[q];
				}
				const double *V = &Vinv[4 * i];
				for (int v = 0; v < 4; v++)
					for (int d = 0; d < 2; d++)
						grad[8 * i + 2 * v + d] = V[2 * d] * fs[2 * v] + V[2 * d + 1] * fs[2 * v + 1];
			}
		}
	}

	// ---------- reconstruction ----------
	/* linearExtrapolate, reconstruction_utils.hpp */
	static double linext(double uc, const double *g, int v, double lim, const double *gp, const double *rcc)
	{
		double uf = uc;
		for (int d = 0; d < 2; d++) uf += lim * g[2 * v + d] * (gp[d] - rcc[d]);
		return uf;
	}

	/* compute_face_values for every reconstruction; up: cell prim, ug: ghost prim,
	 * ufl/ufr: naface x 4 (primitive face values). */
	void face_values(const double *up, const double *ug, const double *grad, double *ufl, double *ufr) const
	{
		const Mesh &M = *m;
		const int ne = M.nelem, nf = M.naface, nb = M.nbface;
		auto nbr_val = [&](int jel, int v) { return jel < ne ? up[4 * jel + v] : ug[4 * (jel - ne) + v]; };
		if (recon == R_NONE) {
			/* LinearUnlimitedReconstruction, areconstruction.cpp:53-103 */
#pragma omp parallel for schedule(static)
			for (int f = 0; f < nf; f++) {
				const int ie = M.intfac[4 * f], je = M.intfac[4 * f + 1];
				for (int v = 0; v < 4; v++) {
					ufl[4 * f + v] = linext(up[4 * ie + v], &grad[8 * ie], v, 1.0, &gr[2 * f], &rc[2 * ie]);
					if (f >= nb) ufr[4 * f + v] = linext(up[4 * je + v], &grad[8 * je], v, 1.0, &gr[2 * f], &rc[2 * je]);
				}
			}
		} else if (recon == R_VANALBADA) {
			/* MUSCLVanAlbada, musclreconstruction.cpp:25-130 (eps 1e-8, k 1/3) */
			const double eps = 1e-8, k = 1.0 / 3.0;
			auto bdiff = [](const double *ri, const double *rj, double ui, double uj, const double *g) {
				double del = 0;
				for (int d = 0; d < 2; d++) del += g[d] * (rj[d] - ri[d]);
				return 2.0 * del - (uj - ui);
			};
			auto recl = [&](double ui, double uj, double dm, double phi) {
				return ui + phi / 4.0 * ((1.0 - k * phi) * dm + (1.0 + k * phi) * (uj - ui));
			};
			auto recr = [&](double ui, double uj, double dp, double phi) {
				return uj - phi / 4.0 * ((1.0 - k * phi) * dp + (1.0 + k * phi) * (uj - ui));
			};
#pragma omp parallel for schedule(static)
			for (int f = 0; f < nf; f++) {
				const int ie = M.intfac[4 * f], je = M.intfac[4 * f + 1];
				if (f < nb) {
					for (int v = 0; v < 4; v++) {
						const double uj = ug[4 * f + v], ui = up[4 * ie + v];
						const double dm = bdiff(&rc[2 * ie], &rcbp[2 * f], ui, uj, &grad[8 * ie + 2 * v]);
						double phl = (2.0 * dm * (uj - ui) + eps) / (dm * dm + (uj - ui) * (uj - ui) + eps);
						if (phl < 0.0) phl = 0.0;
						ufl[4 * f + v] = recl(ui, uj, dm, phl);
					}
				} else {
					for (int v = 0; v < 4; v++) {
						const double ui = up[4 * ie + v], uj = up[4 * je + v];
						const double dm = bdiff(&rc[2 * ie], &rc[2 * je], ui, uj, &grad[8 * ie + 2 * v]);
						const double dp = bdiff(&rc[2 * ie], &rc[2 * je], ui, uj, &grad[8 * je + 2 * v]);
						double phl = (2.0 * dm * (uj - ui) + eps) / (dm * dm + (uj - ui) * (uj - ui) + eps);
						if (phl < 0.0) phl = 0.0;
						double phr = (2 * dp * (uj - ui) + eps) / (dp * dp + (uj - ui) * (uj - ui) + eps);
						if (phr < 0.0) phr = 0.0;
						ufl[4 * f + v] = recl(ui, uj, dm, phl);
						ufr[4 * f + v] = recr(ui, uj, dp, phr);
					}
				}
			}
		} else if (recon == R_WENO) {
			/* WENOReconstruction, limitedlinearreconstruction.cpp:28-105 (gamma 4, eps 1e-5) */
			const double gam = 4.0, lambda = limparam, epsw = 1.0e-5;
#pragma omp parallel for schedule(static)
			for (int ie = 0; ie < ne; ie++) {
				for (int v = 0; v < 4; v++) {
					double wsum = 0, lg[2] = {0, 0};
					{
						const double *g = &grad[8 * ie + 2 * v];
						const double den = std::pow(g[0] * g[0] + g[1] * g[1] + epsw, gam);
						const double w = lambda / den;
						wsum += w;
						for (int d = 0; d < 2; d++) lg[d] += w * g[d];
					}
					for (int j = 0; j < M.nnode[ie]; j++) {
						const int je = M.esuel[4 * ie + j];
						if (je >= ne) continue;
						const double *g = &grad[8 * je + 2 * v];
						const double den = std::pow(g[0] * g[0] + g[1] * g[1] + epsw, gam);
						const double w = 1.0 / den;
						wsum += w;
						for (int d = 0; d < 2; d++) lg[d] += w * g[d];
					}
					for (int d = 0; d < 2; d++) lg[d] /= wsum;
					for (int j = 0; j < M.nnode[ie]; j++) {
						const int f = M.elemface[4 * ie + j], je = M.esuel[4 * ie + j];
						double val = up[4 * ie + v];
						for (int d = 0; d < 2; d++) val += lg[d] * (gr[2 * f + d] - rc[2 * ie + d]);
						if (ie < je) ufl[4 * f + v] = val;
						else ufr[4 * f + v] = val;
					}
				}
			}
		} else {
			/* BarthJespersenLimiter :117-175, VenkatakrishnanLimiter :207-268 */
			const bool venkat = recon == R_VENKATAKRISHNAN;
#pragma omp parallel for schedule(static)
			for (int ie = 0; ie < ne; ie++) {
				const double eps2 = venkat ? std::pow(limparam * clength[ie], 3) : 0.0;
				for (int v = 0; v < 4; v++) {
					double dmin = 0, dmax = 0;
					for (int j = 0; j < M.nnode[ie]; j++) {
						const double d = nbr_val(M.esuel[4 * ie + j], v) - up[4 * ie + v];
						if (d > dmax) dmax = d;
						if (d < dmin) dmin = d;
					}
					double lim = 1.0;
					for (int j = 0; j < M.nnode[ie]; j++) {
						const int f = M.elemface[4 * ie + j];
						const double uf = linext(up[4 * ie + v], &grad[8 * ie], v, 1.0, &gr[2 * f], &rc[2 * ie]);
						double phi;
						if (venkat) {
							const double dm = uf - up[4 * ie + v];
							const double dp = dm < 0 ? dmin : dmax;
							phi = (dp * dp + 2 * dp * dm + eps2) / (dp * dp + dp * dm + 2 * dm * dm + eps2);
						} else {
							const double diff = uf - up[4 * ie + v];
							if (diff > 0) phi = 1 < dmax / diff ? 1 : dmax / diff;
							else if (diff < 0) phi = 1 < dmin / diff ? 1 : dmin / diff;
							else phi = 1;
						}
						if (phi < lim) lim = phi;
					}
					for (int j = 0; j < M.nnode[ie]; j++) {
						const int f = M.elemface[4 * ie + j], je = M.esuel[4 * ie + j];
						const double val = linext(up[4 * ie + v], &grad[8 * ie], v, lim, &gr[2 * f], &rc[2 * ie]);
						if (ie < je) ufl[4 * f + v] = val;
						else ufr[4 * f + v] = val;
					}
				}
			}
		}
	}

	// ---------- residual (flow_spatial.cpp:488-816) ----------
	struct Work {
		std::vector<double> uleft, uright, ubcell, up, grad, fflux, spec;
	};

	void compute_viscous_flux(int f, const double *ucl, const double *ucr, const double *gl, const double *gr_,
	                          const double *ul, const double *ur, const double *rcr, double *vflux) const
	{
		/* FlowFV::compute_viscous_flux, flow_spatial.cpp:348-395 */
		double uctl[4], uctr[4], gtl[8], gtr[8], gl2[8], gr2[8];
		// GradBlock_t is column-major 2 x 4; the viscous routines take NDIM x NVARS row-major
		for (int d = 0; d < 2; d++)
			for (int v = 0; v < 4; v++) {
				gl2[d * 4 + v] = order2 ? gl[2 * v + d] : 0.0;
				gr2[d * 4 + v] = order2 ? gr_[2 * v + d] : 0.0;
			}
		prim2_states_grads(P, order2, ucl, ucr, gl2, gr2, uctl, uctr, gtl, gtr);
		if (!order2)
			for (int k = 0; k < 8; k++) { gtl[k] = 0; gtr[k] = 0; }
		double grad[2][4];
		face_gradient_modavg(&rc[2 * m->intfac[4 * f]], rcr, uctl, uctr, gtl, gtr, grad);
		viscous_flux(P, constvisc, &m->facemetric[3 * f], grad, ul, ur, vflux);
	}

	/* FlowFV::compute_residual: r += -R(u); dt (if requested) = A/sum(specrad). */
	void residual(const double *u, double *r, bool gettimesteps, double *dt, Work &w) const
	{
		const Mesh &M = *m;
		const int ne = M.nelem, nf = M.naface, nb = M.nbface;
		w.uleft.assign(4 * (size_t)nf, 0.0);
		w.uright.assign(4 * (size_t)nf, 0.0);
		w.ubcell.assign(4 * (size_t)nb, 0.0);
		double *ul = w.uleft.data(), *ur = w.uright.data();
		for (int f = 0; f < nb; f++)
			for (int v = 0; v < 4; v++) ul[4 * f + v] = u[4 * M.intfac[4 * f] + v];
		if (order2) {
			for (int f = 0; f < nb; f++) boundary_state(f, &ul[4 * f], &ur[4 * f]);
			w.up.assign(4 * (size_t)ne, 0.0);
			for (int f = 0; f < nb; f++) {
				for (int v = 0; v < 4; v++) w.ubcell[4 * f + v] = ur[4 * f + v];
				prim_from_cons(P, &ur[4 * f], &ur[4 * f]);
			}
#pragma omp parallel for schedule(static)
			for (int i = 0; i < ne; i++) prim_from_cons(P, &u[4 * i], &w.up[4 * i]);
			std::vector<double> ug(ur, ur + 4 * nb);
			w.grad.assign(8 * (size_t)ne, 0.0);
			gradients(w.up.data(), ug.data(), w.grad.data());
			face_values(w.up.data(), ug.data(), w.grad.data(), ul, ur);
#pragma omp parallel for schedule(static)
			for (int f = 0; f < nf; f++) {
				cons_from_prim(P, &ul[4 * f], &ul[4 * f]);
				if (f >= nb) cons_from_prim(P, &ur[4 * f], &ur[4 * f]);
			}
		} else {
#pragma omp parallel for schedule(static)
			for (int f = nb; f < nf; f++)
				for (int v = 0; v < 4; v++) {
					ul[4 * f + v] = u[4 * M.intfac[4 * f] + v];
					ur[4 * f + v] = u[4 * M.intfac[4 * f + 1] + v];
				}
		}
		for (int f = 0; f < nb; f++) boundary_state(f, &ul[4 * f], &ur[4 * f]);
		const double *ug_pb = order2 ? w.ubcell.data() : ur;  // indexed 4*f for f < nb
		/* compute_fluxes, flow_spatial.cpp:488-563 and compute_max_timestep :565-634 */
		w.fflux.assign(4 * (size_t)nf, 0.0);
		w.spec.assign(2 * (size_t)nf, 0.0);
#pragma omp parallel for schedule(static)
		for (int f = 0; f < nf; f++) {
			const double *n = &M.facemetric[3 * f];
			const double len = n[2];
			const int le = M.intfac[4 * f], re = M.intfac[4 * f + 1];
			double fl[4] = {0, 0, 0, 0};
			numerical_flux(flux, P, &ul[4 * f], &ur[4 * f], n, fl);
			for (int v = 0; v < 4; v++) fl[v] *= len;
			if (viscous) {
				const bool isb = f < nb;
				const double *rcr = isb ? &rcbp[2 * f] : &rc[2 * re];
				const double *ucr = isb ? &ug_pb[4 * f] : &u[4 * re];
				const double *gl = order2 ? &w.grad[8 * le] : nullptr;
				const double *grr = order2 ? (isb ? &w.grad[8 * le] : &w.grad[8 * re]) : nullptr;
				double vf[4];
				compute_viscous_flux(f, &u[4 * le], ucr, gl, grr, &ul[4 * f], &ur[4 * f], rcr, vf);
				for (int v = 0; v < 4; v++) fl[v] += vf[v] * len;
			}
			for (int v = 0; v < 4; v++) w.fflux[4 * f + v] = fl[v];
			if (gettimesteps) {
				const double *a = &ul[4 * f], *b = &ur[4 * f];
				const double ci = sound_speed(P, a[0], pressure_from_cons(P, a));
				const double cj = sound_speed(P, b[0], pressure_from_cons(P, b));
				const double vni = dot2n(&a[1], n) / a[0], vnj = dot2n(&b[1], n) / b[0];
				double si = (std::fabs(vni) + ci) * len, sj = (std::fabs(vnj) + cj) * len;
				if (viscous) {
					double mui, muj;
					if (constvisc) { mui = muj = 1.0 / P.Reinf; }
					else {
						mui = sutherland(P, temperature(P, a[0], pressure_from_cons(P, a)));
						muj = sutherland(P, temperature(P, b[0], pressure_from_cons(P, b)));
					}
					const double coi = std::max(4.0 / (3 * a[0]), P.g / a[0]);
					const double coj = std::max(4.0 / (3 * b[0]), P.g / b[0]);
					si += coi * mui / P.Pr * len * len / M.area[le];
					if (re < ne) sj += coj * muj / P.Pr * len * len / M.area[re];
				}
				w.spec[2 * f] = si;
				w.spec[2 * f + 1] = sj;
			}
		}
#pragma omp parallel for schedule(static)
		for (int i = 0; i < ne; i++) {
			double acc[4] = {0, 0, 0, 0}, integ = 0;
			for (int k = M.cf_ptr[i]; k < M.cf_ptr[i + 1]; k++) {
				const int f = M.cf_face[k];
				const double s = M.cf_side[k] ? 1.0 : -1.0;
				for (int v = 0; v < 4; v++) acc[v] += s * w.fflux[4 * f + v];
				integ += w.spec[2 * f + M.cf_side[k]];
			}
			for (int v = 0; v < 4; v++) r[4 * i + v] += acc[v];
			if (gettimesteps) dt[i] = M.area[i] / integ;
		}
	}

	/* FlowFV_base::getGradients, flow_spatial.cpp:95-112: conserved-variable
	 * gradients with ghost states from cell values. */
	void conserved_gradients(const double *u, double *grad) const
	{
		const Mesh &M = *m;
		std::vector<double> ug(4 * (size_t)M.nbface);
		for (int f = 0; f < M.nbface; f++) boundary_state(f, &u[4 * M.intfac[4 * f]], &ug[4 * f]);
		gradients(u, ug.data(), grad);
	}

	// ---------- Jacobian blocks (flow_spatial.cpp:818-875) ----------
	/* Jacobian-flux (and thin-layer viscous flux) derivatives; L = -dF/dul*len,
	 * U = dF/dur*len (row-major 4x4). */
	int face_flux_derivs(int f, const double *ul, const double *ur, const double *rcr, double *L, double *U) const
	{
		typedef Dual<8> D8;
		D8 a[4], b[4], F[4];
		for (int i = 0; i < 4; i++) {
			a[i] = D8(ul[i]); a[i].d[i] = 1.0;
			b[i] = D8(ur[i]); b[i].d[4 + i] = 1.0;
		}
		const double *n = &m->facemetric[3 * f];
		if (fluxjac == F_VANLEER || fluxjac == F_AUSMPLUS) return 2;
		numerical_flux(fluxjac, P, a, b, n, F);
		if (viscous) {
			D8 vf[4];
			viscous_flux_thinlayer(P, constvisc, n, &rc[2 * m->intfac[4 * f]], rcr, a, b, vf);
			for (int i = 0; i < 4; i++) F[i] += vf[i];
		}
		for (int i = 0; i < 4; i++)
			for (int k = 0; k < 4; k++) {
				L[4 * i + k] = -F[i].d[k];
				U[4 * i + k] = F[i].d[4 + k];
			}
		return 0;
	}

	/* compute_local_jacobian_interior (:818-839) */
	int local_jac_interior(int f, const double *ul, const double *ur, double *L, double *U) const
	{
		const double len = m->facemetric[3 * f + 2];
		if (int e = face_flux_derivs(f, ul, ur, &rc[2 * m->intfac[4 * f + 1]], L, U)) return e;
		for (int k = 0; k < 16; k++) { L[k] *= len; U[k] *= len; }
		return 0;
	}

	/* compute_local_jacobian_boundary (:841-875): left = len*(L - U*dghost/dul) */
	int local_jac_boundary(int f, const double *ul, double *left) const
	{
		const double len = m->facemetric[3 * f + 2];
		double gs[4], G[16], L[16], U[16];
		if (int e = ghost_jacobian(P, bc_of_face(f), uinf, ul, &m->facemetric[3 * f], gs, G)) return e;
		if (int e = face_flux_derivs(f, ul, gs, &rcbp[2 * f], L, U)) return e;
		for (int i = 0; i < 4; i++)
			for (int k = 0; k < 4; k++) {
				double s = 0;
				for (int j = 0; j < 4; j++) s += U[4 * i + j] * G[4 * j + k];
				left[4 * i + k] = len * (L[4 * i + k] - s);
			}
		return 0;
	}
};

// ====================== block sparse matrix (BAIJ, bs=4) =====================

/* Rows sorted by column, diagonal included; preallocation nfael+1 blocks/row
 * (alinalg.cpp:43-85). */
struct BSR {
	int n = 0;
	std::vector<int> rowptr, col, diag;  // diag[i] = position of (i,i)
	std::vector<double> val;             // nnzb x 16
	void setup(const Mesh &M)
	{
		n = M.nelem;
		rowptr.assign(n + 1, 0);
		col.clear();
		diag.assign(n, -1);
		for (int i = 0; i < n; i++) {
			std::vector<int> c{i};
			for (int j = 0; j < M.nnode[i]; j++)
				if (M.esuel[4 * i + j] >= 0 && M.esuel[4 * i + j] < n) c.push_back(M.esuel[4 * i + j]);
			std::sort(c.begin(), c.end());
			for (int x : c) {
				if (x == i) diag[i] = (int)col.size();
				col.push_back(x);
			}
			rowptr[i + 1] = (int)col.size();
		}
		val.assign(16 * col.size(), 0.0);
	}
	int find(int i, int j) const
	{
		for (int k = rowptr[i]; k < rowptr[i + 1]; k++)
			if (col[k] == j) return k;
		return -1;
	}
	void zero() { std::fill(val.begin(), val.end(), 0.0); }
	void add(int i, int j, const double *b, double s)
	{
		const int k = find(i, j);
		for (int q = 0; q < 16; q++) val[16 * k + q] += s * b[q];
	}
	void matvec(const double *x, double *y) const
	{
#pragma omp parallel for schedule(static)
		for (int i = 0; i < n; i++) {
			double acc[4] = {0, 0, 0, 0};
			for (int k = rowptr[i]; k < rowptr[i + 1]; k++) {
				const double *b = &val[16 * k];
				const double *xx = &x[4 * col[k]];
				for (int r = 0; r < 4; r++)
					for (int c = 0; c < 4; c++) acc[r] += b[4 * r + c] * xx[c];
			}
			for (int r = 0; r < 4; r++) y[4 * i + r] = acc[r];
		}
	}
};

/* Spatial::assemble_jacobian, aspatial.cpp:242-340 (ADD_VALUES into zeroed M). */
inline int assemble_jacobian(const Disc &D, const double *u, BSR &A)
{
	const Mesh &M = *D.m;
	const int nf = M.naface, nb = M.nbface;
	std::vector<double> blk(32 * (size_t)nf);
	int err = 0;
#pragma omp parallel for schedule(static) reduction(| : err)
	for (int f = 0; f < nf; f++) {
		const int l = M.intfac[4 * f], r = M.intfac[4 * f + 1];
		if (f < nb)
			err |= D.local_jac_boundary(f, &u[4 * l], &blk[32 * f]);
		else
			err |= D.local_jac_interior(f, &u[4 * l], &u[4 * r], &blk[32 * f], &blk[32 * f + 16]);
	}
	if (err) return err;
	// off-diagonal blocks are each touched by exactly one face
#pragma omp parallel for schedule(static)
	for (int f = nb; f < nf; f++) {
		const int l = M.intfac[4 * f], r = M.intfac[4 * f + 1];
		const int krl = A.find(r, l), klr = A.find(l, r);
		for (int q = 0; q < 16; q++) {
			A.val[16 * krl + q] += blk[32 * f + q];
			A.val[16 * klr + q] += blk[32 * f + 16 + q];
		}
	}
	// diagonal: gathered per cell in ascending face order
#pragma omp parallel for schedule(static)
	for (int i = 0; i < M.nelem; i++) {
		double d[16] = {0};
		for (int k = M.cf_ptr[i]; k < M.cf_ptr[i + 1]; k++) {
			const int f = M.cf_face[k];
			const double *b = f < nb ? &blk[32 * f] : (M.cf_side[k] ? &blk[32 * f + 16] : &blk[32 * f]);
			for (int q = 0; q < 16; q++) d[q] -= b[q];
		}
		for (int q = 0; q < 16; q++) A.val[16 * A.diag[i] + q] += d[q];
	}
	return 0;
}

// ============================ small dense helpers ============================

inline bool inv4(const double *a, double *out)
{
	double m[4][8];
	for (int i = 0; i < 4; i++)
		for (int j = 0; j < 8; j++) m[i][j] = j < 4 ? a[4 * i + j] : (j - 4 == i ? 1.0 : 0.0);
	for (int c = 0; c < 4; c++) {
		int p = c;
		for (int r = c + 1; r < 4; r++)
			if (std::fabs(m[r][c]) > std::fabs(m[p][c])) p = r;
		if (m[p][c] == 0.0) return false;
		if (p != c)
			for (int j = 0; j < 8; j++) std::swap(m[p][j], m[c][j]);
		const double iv = 1.0 / m[c][c];
		for (int j = 0; j < 8; j++) m[c][j] *= iv;
		for (int r = 0; r < 4; r++)
			if (r != c) {
				const double fct = m[r][c];
				for (int j = 0; j < 8; j++) m[r][j] -= fct * m[c][j];
			}
	}
	for (int i = 0; i < 4; i++)
		for (int j = 0; j < 4; j++) out[4 * i + j] = m[i][j + 4];
	return true;
}
inline void mm4(const double *a, const double *b, double *c)
{
	for (int i = 0; i < 4; i++)
		for (int j = 0; j < 4; j++) {
			double s = 0;
			for (int k = 0; k < 4; k++) s += a[4 * i + k] * b[4 * k + j];
			c[4 * i + j] = s;
		}
}
inline void mv4(const double *a, const double *x, double *y)
{
	for (int i = 0; i < 4; i++) y[i] = a[4 * i] * x[0] + a[4 * i + 1] * x[1] + a[4 * i + 2] * x[2] + a[4 * i + 3] * x[3];
}

// ============================== preconditioners ==============================

enum { PC_NONE = 0, PC_JACOBI = 1, PC_SGS = 2, PC_ILU0 = 3 };

/* Preconditioners on the BAIJ matrix in a given elimination order (pos[i] =
 * position of cell i).  Natural order reproduces PETSc's sequential
 * -sub_pc_type ilu / -pc_type sor on the (RCM-reordered) matrix. */
struct Precond {
	int type = PC_NONE;
	const BSR *A = nullptr;
	std::vector<int> order, pos;   // elimination order
	std::vector<double> F;         // factored values (ILU0) or copy
	std::vector<double> Dinv;      // inverted diagonal blocks (Jacobi/SGS) or inverted U_ii (ILU0)

	int setup(const BSR &Am, int t, const int *ord)
	{
		A = &Am;
		type = t;
		const int n = Am.n;
		order.resize(n);
		pos.resize(n);
		for (int i = 0; i < n; i++) order[i] = ord ? ord[i] : i;
		for (int i = 0; i < n; i++) pos[order[i]] = i;
		Dinv.assign(16 * (size_t)n, 0.0);
		if (type == PC_JACOBI || type == PC_SGS) {
			for (int i = 0; i < n; i++)
				if (!inv4(&Am.val[16 * Am.diag[i]], &Dinv[16 * i])) return 4;
		} else if (type == PC_ILU0) {
			F = Am.val;
			for (int oi = 0; oi < n; oi++) {
				const int i = order[oi];
				// L-neighbours of i sorted by elimination position
				std::vector<std::pair<int, int>> lk;
				for (int k = Am.rowptr[i]; k < Am.rowptr[i + 1]; k++)
					if (pos[Am.col[k]] < oi) lk.push_back({pos[Am.col[k]], k});
				std::sort(lk.begin(), lk.end());
				for (auto &pk : lk) {
					const int kk = pk.second, kc = Am.col[kk];
					double t16[16];
					mm4(&F[16 * kk], &Dinv[16 * kc], t16);
					std::memcpy(&F[16 * kk], t16, sizeof(t16));
					for (int j = Am.rowptr[i]; j < Am.rowptr[i + 1]; j++) {
						const int jc = Am.col[j];
						if (pos[jc] <= pos[kc]) continue;
						const int kj = Am.find(kc, jc);
						if (kj < 0) continue;
						double p16[16];
						mm4(&F[16 * kk], &F[16 * kj], p16);
						for (int q = 0; q < 16; q++) F[16 * j + q] -= p16[q];
					}
				}
				if (!inv4(&F[16 * Am.diag[i]], &Dinv[16 * i])) return 4;
			}
		}
		return 0;
	}

	void apply(const double *r, double *z) const
	{
		const int n = A->n;
		const BSR &Am = *A;
		if (type == PC_NONE) {
			std::memcpy(z, r, sizeof(double) * 4 * n);
		} else if (type == PC_JACOBI) {
#pragma omp parallel for schedule(static)
			for (int i = 0; i < n; i++) mv4(&Dinv[16 * i], &r[4 * i], &z[4 * i]);
		} else {
			const std::vector<double> &V = type == PC_ILU0 ? F : Am.val;
			std::vector<double> y(4 * (size_t)n);
			for (int oi = 0; oi < n; oi++) {
				const int i = order[oi];
				double s[4] = {r[4 * i], r[4 * i + 1], r[4 * i + 2], r[4 * i + 3]};
				for (int k = Am.rowptr[i]; k < Am.rowptr[i + 1]; k++)
					if (pos[Am.col[k]] < oi) {
						double t[4];
						mv4(&V[16 * k], &y[4 * Am.col[k]], t);
						for (int q = 0; q < 4; q++) s[q] -= t[q];
					}
				if (type == PC_SGS) mv4(&Dinv[16 * i], s, &y[4 * i]);
				else for (int q = 0; q < 4; q++) y[4 * i + q] = s[q];
			}
			for (int oi = n - 1; oi >= 0; oi--) {
				const int i = order[oi];
				double s[4] = {0, 0, 0, 0};
				for (int k = Am.rowptr[i]; k < Am.rowptr[i + 1]; k++)
					if (pos[Am.col[k]] > oi) {
						double t[4];
						mv4(&V[16 * k], &z[4 * Am.col[k]], t);
						for (int q = 0; q < 4; q++) s[q] += t[q];
					}
				if (type == PC_SGS) {
					double t[4];
					mv4(&Dinv[16 * i], s, t);
					for (int q = 0; q < 4; q++) z[4 * i + q] = y[4 * i + q] - t[q];
				} else {
					double t[4];
					for (int q = 0; q < 4; q++) t[q] = y[4 * i + q] - s[q];
					mv4(&Dinv[16 * i], t, &z[4 * i]);
				}
			}
		}
	}
};

// ================================= FGMRES ===================================

/* dot product in a fixed order whatever the thread count: sums of blocks of
 * 4096 entries (in parallel), then the block sums in order */
inline double dotv(const double *a, const double *b, size_t n)
{
	constexpr size_t BLK = 4096;
	const long nb = (long)((n + BLK - 1) / BLK);
	std::vector<double> part(nb > 0 ? nb : 1, 0.0);
#pragma omp parallel for schedule(static)
	for (long k = 0; k < nb; k++) {
		const size_t i1 = std::min(n, (size_t)(k + 1) * BLK);
		double s = 0;
		for (size_t i = (size_t)k * BLK; i < i1; i++) s += a[i] * b[i];
		part[k] = s;
	}
	double s = 0;
	for (long k = 0; k < nb; k++) s += part[k];
	return s;
}

/* Right-preconditioned flexible GMRES(m), classical Gram-Schmidt, x0 = 0.
 * op(x, y) applies the operator.  Returns the iteration count. */
template <class Op>
int fgmres(Op op, const Precond &pc, const double *b, double *x, size_t n, int restart, int maxit, double rtol,
           double *final_rnorm)
{
	std::fill(x, x + n, 0.0);
	const double bnorm = std::sqrt(dotv(b, b, n));
	if (final_rnorm) *final_rnorm = bnorm;
	if (bnorm == 0.0) return 0;
	const double target = rtol * bnorm;
	int its = 0;
	std::vector<double> r(b, b + n), w(n);
	double beta = bnorm;
	while (its < maxit) {
		const int mres = std::min(restart, maxit - its);
		std::vector<std::vector<double>> V(mres + 1, std::vector<double>(n)), Z(mres, std::vector<double>(n));
		std::vector<double> H((mres + 1) * mres, 0.0), cs(mres), sn(mres), g(mres + 1, 0.0);
		for (size_t i = 0; i < n; i++) V[0][i] = r[i] / beta;
		g[0] = beta;
		int k = 0;
		for (; k < mres; k++) {
			pc.apply(V[k].data(), Z[k].data());
			op(Z[k].data(), w.data());
			// classical Gram-Schmidt
			std::vector<double> h(k + 1);
			for (int j = 0; j <= k; j++) h[j] = dotv(V[j].data(), w.data(), n);
			for (int j = 0; j <= k; j++) {
				const double hj = h[j];
				const double *vj = V[j].data();
#pragma omp parallel for schedule(static)
				for (long i = 0; i < (long)n; i++) w[i] -= hj * vj[i];
			}
			const double hn = std::sqrt(dotv(w.data(), w.data(), n));
			for (int j = 0; j <= k; j++) H[j * mres + k] = h[j];
			H[(k + 1) * mres + k] = hn;
			if (hn != 0.0)
				for (size_t i = 0; i < n; i++) V[k + 1][i] = w[i] / hn;
			for (int j = 0; j < k; j++) {
				const double a = H[j * mres + k], bb = H[(j + 1) * mres + k];
				H[j * mres + k] = cs[j] * a + sn[j] * bb;
				H[(j + 1) * mres + k] = -sn[j] * a + cs[j] * bb;
			}
			const double a = H[k * mres + k], bb = H[(k + 1) * mres + k];
			const double den = std::sqrt(a * a + bb * bb);
			cs[k] = a / den;
			sn[k] = bb / den;
			H[k * mres + k] = den;
			H[(k + 1) * mres + k] = 0.0;
			g[k + 1] = -sn[k] * g[k];
			g[k] = cs[k] * g[k];
			its++;
			if (std::fabs(g[k + 1]) <= target || hn == 0.0) { k++; break; }
		}
		// solve H y = g (upper triangular k x k)
		std::vector<double> y(k);
		for (int i = k - 1; i >= 0; i--) {
			double s = g[i];
			for (int j = i + 1; j < k; j++) s -= H[i * mres + j] * y[j];
			y[i] = s / H[i * mres + i];
		}
		for (int j = 0; j < k; j++)
			for (size_t i = 0; i < n; i++) x[i] += y[j] * Z[j][i];
		const double rn = std::fabs(g[k]);
		if (final_rnorm) *final_rnorm = rn;
		if (rn <= target || its >= maxit) break;
		// restart: r = b - A x
		op(x, w.data());
		for (size_t i = 0; i < n; i++) r[i] = b[i] - w[i];
		beta = std::sqrt(dotv(r.data(), r.data(), n));
	}
	return its;
}

// ========================= steady backward Euler ============================

struct SolverCfg {
	double cflmin = 10, cflmax = 1000, tol = 1e-10;
	int maxiter = 1000;
	int abs_tol = 1;        // 1: ||R|| < tol (absolute); 0: relative to step 0 (reference)
	int pc = PC_ILU0;
	int restart = 30, lin_maxit = 30;
	double lin_rtol = 0.1;
	int matrix_free = 0;
	double mf_eps = 1e-7;
	int nl_update = 0;      // 0 full, 1 robust_flow (FlowSimpleUpdate), 2 robust_flow with bounded change
	double min_relax = 0.2;
};

struct SolveStats {
	int steps = 0, lin_iters = 0, status = 0;
	double res0 = 0, res = 0, cfl = 0;
};

/* expResidualRamp, aodesolver.cpp:110-120 */
inline double exp_residual_ramp(double cflmin, double cflmax, double prevcfl, double ratio, double up, double down)
{
	const double nc = ratio > 1.0 ? prevcfl * std::pow(ratio, up) : prevcfl * std::pow(ratio, down);
	if (nc < cflmin) return cflmin;
	if (nc > cflmax) return cflmax;
	return nc;
}

/* FlowSimpleUpdate::getLocalRelaxationFactor, nonlinearrelaxation.cpp:25-38 */
inline double relax_factor(const Phys &P, double minf, const double *du, const double *u, int mode)
{
	const double p = pressure_from_cons(P, u);
	const double dp = std::fabs(delta_pressure(P, u, du)) / p;
	const double dr = std::fabs(du[0]) / u[0];
	const double dl = std::max(dp, dr);
	double om = minf;
	if (dl < 1.0 - minf) om = 1.0 - dl;
	// mode 2 (not in the reference): above the threshold the factor also
	// keeps the relative density / pressure change at minf (1 - minf), and it
	// is halved until the updated density and pressure (the exact ones, which
	// the linearised change misses when the momentum changes a lot) stay above
	// minf times their old values
	else if (mode == 2) om = minf * (1.0 - minf) / dl;
	if (mode == 2) {
		for (int k = 0; k < 40; k++) {
			double un[4];
			for (int q = 0; q < 4; q++) un[q] = u[q] + om * du[q];
			if (un[0] >= minf * u[0] && pressure_from_cons(P, un) >= minf * p) break;
			om *= 0.5;
		}
	}
	return om;
}

/* SteadyBackwardEulerSolver::solve, aodesolver.cpp:363-638 */
inline int steady_solve(const Disc &D, const SolverCfg &c, double *u, SolveStats &st, const int *pc_order,
                        double *history /* 3 x maxiter: res, cfl, linits */)
{
	const Mesh &M = *D.m;
	const int ne = M.nelem;
	const size_t n = 4 * (size_t)ne;
	std::vector<double> r(n), du(n), dtm(ne), aux(n), yg(n);
	BSR A;
	A.setup(M);
	Disc::Work w, w2;
	double cfl = 0, resi = 1.0, resiold = 1.0, initres = 1.0;
	int step = 0;
	st = SolveStats();
	while (step < c.maxiter) {
		if (step > 0) {
			if (c.abs_tol ? (resi <= c.tol) : (resi / initres <= c.tol)) break;
		}
		std::fill(r.begin(), r.end(), 0.0);
		D.residual(u, r.data(), true, dtm.data(), w);
		A.zero();
		if (int e = assemble_jacobian(D, u, A)) { st.status = e; return e; }
		cfl = exp_residual_ramp(c.cflmin, c.cflmax, cfl, resiold / resi, 0.25, 0.3);
		/* addPseudoTimeTerm, aodesolver.cpp:300-329 */
		for (int i = 0; i < ne; i++) {
			dtm[i] = M.area[i] / (cfl * dtm[i]);
			for (int q = 0; q < 4; q++) A.val[16 * A.diag[i] + 5 * q] += dtm[i];
		}
		Precond pc;
		if (int e = pc.setup(A, c.pc, pc_order)) { st.status = e; return e; }
		int its;
		if (c.matrix_free) {
			/* MatrixFreeSpatialJacobian::apply, alinalg.cpp:143-237 */
			auto op = [&](const double *x, double *y) {
				const double xn = std::sqrt(dotv(x, x, n));
				const double pm = c.mf_eps / xn;
				for (size_t i = 0; i < n; i++) { yg[i] = 0; aux[i] = u[i] + pm * x[i]; }
				D.residual(aux.data(), yg.data(), false, nullptr, w2);
				for (int i = 0; i < ne; i++)
					for (int q = 0; q < 4; q++)
						y[4 * i + q] = dtm[i] * x[4 * i + q] + (-yg[4 * i + q] + r[4 * i + q]) / pm;
			};
			its = fgmres(op, pc, r.data(), du.data(), n, c.restart, c.lin_maxit, c.lin_rtol, nullptr);
		} else {
			auto op = [&](const double *x, double *y) { A.matvec(x, y); };
			its = fgmres(op, pc, r.data(), du.data(), n, c.restart, c.lin_maxit, c.lin_rtol, nullptr);
		}
		st.lin_iters += its;
		for (int i = 0; i < ne; i++) {
			const double om = c.nl_update ? relax_factor(D.P, c.min_relax, &du[4 * i], &u[4 * i], c.nl_update) : 1.0;
			for (int q = 0; q < 4; q++) u[4 * i + q] += om * du[4 * i + q];
		}
		double rn2 = 0;
		for (int i = 0; i < ne; i++) rn2 += r[4 * i + 3] * r[4 * i + 3] * M.area[i];
		resiold = resi;
		resi = std::sqrt(rn2);
		if (history) {
			history[3 * step] = resi;
			history[3 * step + 1] = cfl;
			history[3 * step + 2] = its;
		}
		if (!std::isfinite(resi)) { st.status = 5; st.steps = step + 1; st.res = resi; return 5; }
		if (step == 0) initres = resi;
		step++;
	}
	st.steps = step;
	st.res0 = initres;
	st.res = resi;
	st.cfl = cfl;
	const bool conv = c.abs_tol ? (resi <= c.tol) : (resi / initres <= c.tol);
	st.status = conv ? 0 : 6;
	return st.status;
}

}  // namespace orc

// ================================ C API =====================================

using namespace orc;

extern "C" {

void *orc_mesh_create(int npoin, const double *coords, int nelem, const int *nnode, const int *inpoel, int nbface,
                      const int *bface, const int *btag)
{
	Mesh *m = new Mesh();
	m->npoin = npoin; m->nelem = nelem; m->nbface = nbface;
	m->coords.assign(coords, coords + 2 * (size_t)npoin);
	m->nnode.assign(nnode, nnode + nelem);
	m->inpoel.assign(inpoel, inpoel + 4 * (size_t)nelem);
	m->bface.assign(bface, bface + 2 * (size_t)nbface);
	m->btag.assign(btag, btag + nbface);
	if (m->build()) { delete m; return nullptr; }
	return m;
}
void orc_mesh_destroy(void *h) { delete (Mesh *)h; }
/* out: nelem, nbface, ninface, naface */
void orc_mesh_counts(const void *h, int *out)
{
	const Mesh *m = (const Mesh *)h;
	out[0] = m->nelem; out[1] = m->nbface; out[2] = m->ninface; out[3] = m->naface;
}
void orc_mesh_arrays(const void *h, int *intfac, int *esuel, double *area, double *facemetric)
{
	const Mesh *m = (const Mesh *)h;
	if (intfac) std::memcpy(intfac, m->intfac.data(), sizeof(int) * m->intfac.size());
	if (esuel) std::memcpy(esuel, m->esuel.data(), sizeof(int) * m->esuel.size());
	if (area) std::memcpy(area, m->area.data(), sizeof(double) * m->area.size());
	if (facemetric) std::memcpy(facemetric, m->facemetric.data(), sizeof(double) * m->facemetric.size());
}

/* phys: gamma, Minf, Tinf, Reinf, Pr, aoa; flags: viscous, constvisc, order2;
 * schemes: flux, fluxjac, gradient, reconstruction; bcs: nbc x (tag, type); bcvals: nbc x 2 */
void *orc_disc_create(const void *mesh, const double *phys, const int *flags, const int *schemes, double limparam,
                      int nbc, const int *bcs, const double *bcvals)
{
	Disc *d = new Disc();
	d->m = (const Mesh *)mesh;
	d->P.g = phys[0]; d->P.Minf = phys[1]; d->P.Tinf = phys[2]; d->P.Reinf = phys[3]; d->P.Pr = phys[4];
	d->aoa = phys[5];
	d->viscous = flags[0]; d->constvisc = flags[1]; d->order2 = flags[2];
	d->flux = schemes[0]; d->fluxjac = schemes[1]; d->gradscheme = schemes[2]; d->recon = schemes[3];
	d->limparam = limparam;
	for (int b = 0; b < nbc; b++) {
		BCSpec s;
		s.type = bcs[2 * b + 1];
		s.vals[0] = bcvals[2 * b]; s.vals[1] = bcvals[2 * b + 1];
		d->bcs[bcs[2 * b]] = s;
	}
	if (d->setup()) { delete d; return nullptr; }
	return d;
}
void orc_disc_destroy(void *h) { delete (Disc *)h; }
void orc_set_threads(int n)
{
#ifdef _OPENMP
	omp_set_num_threads(n);
#endif
	(void)n;
}
int orc_max_threads()
{
#ifdef _OPENMP
	return omp_get_max_threads();
#else
	return 1;
#endif
}
void orc_freestream(const void *h, double *uinf)
{
	const Disc *d = (const Disc *)h;
	for (int i = 0; i < 4; i++) uinf[i] = d->uinf[i];
}
void orc_geometry(const void *h, double *rc, double *rcbp, double *gr)
{
	const Disc *d = (const Disc *)h;
	if (rc) std::memcpy(rc, d->rc.data(), sizeof(double) * d->rc.size());
	if (rcbp) std::memcpy(rcbp, d->rcbp.data(), sizeof(double) * d->rcbp.size());
	if (gr) std::memcpy(gr, d->gr.data(), sizeof(double) * d->gr.size());
}

/* r += -R(u); dt written if dt != NULL */
int orc_residual(const void *h, const double *u, double *r, double *dt)
{
	const Disc *d = (const Disc *)h;
	Disc::Work w;
	d->residual(u, r, dt != nullptr, dt, w);
	return 0;
}
/* primitive-variable gradients as used by the residual, and the face values */
int orc_residual_internals(const void *h, const double *u, double *grad, double *uleft, double *uright)
{
	const Disc *d = (const Disc *)h;
	Disc::Work w;
	std::vector<double> r(4 * (size_t)d->nelem(), 0.0);
	d->residual(u, r.data(), false, nullptr, w);
	if (grad && d->order2) std::memcpy(grad, w.grad.data(), sizeof(double) * w.grad.size());
	if (uleft) std::memcpy(uleft, w.uleft.data(), sizeof(double) * w.uleft.size());
	if (uright) std::memcpy(uright, w.uright.data(), sizeof(double) * w.uright.size());
	return 0;
}
/* per cell: sum over its faces of |F_k * len| (max over k), the scale the
 * residual parity metric is normalised by */
int orc_flux_scale(const void *h, const double *u, double *scale)
{
	const Disc *d = (const Disc *)h;
	Disc::Work w;
	std::vector<double> r(4 * (size_t)d->nelem(), 0.0);
	d->residual(u, r.data(), false, nullptr, w);
	const Mesh &M = *d->m;
	for (int i = 0; i < M.nelem; i++) {
		double s[4] = {0, 0, 0, 0};
		for (int k = M.cf_ptr[i]; k < M.cf_ptr[i + 1]; k++)
			for (int v = 0; v < 4; v++) s[v] += std::fabs(w.fflux[4 * M.cf_face[k] + v]);
		scale[i] = std::max(std::max(s[0], s[1]), std::max(s[2], s[3]));
	}
	return 0;
}
int orc_conserved_gradients(const void *h, const double *u, double *grad)
{
	((const Disc *)h)->conserved_gradients(u, grad);
	return 0;
}

/* Jacobian in BAIJ form; rowptr (nelem+1), col (nnzb), val (nnzb*16).
 * Call with val == NULL to get nnzb in *nnzb. */
int orc_jacobian(const void *h, const double *u, int *nnzb, int *rowptr, int *col, double *val)
{
	const Disc *d = (const Disc *)h;
	BSR A;
	A.setup(*d->m);
	*nnzb = (int)A.col.size();
	if (!val) return 0;
	if (int e = assemble_jacobian(*d, u, A)) return e;
	std::memcpy(rowptr, A.rowptr.data(), sizeof(int) * A.rowptr.size());
	std::memcpy(col, A.col.data(), sizeof(int) * A.col.size());
	std::memcpy(val, A.val.data(), sizeof(double) * A.val.size());
	return 0;
}

/* Median wall time in seconds of `reps` calls (after one untimed call) of each
 * oracle kernel at state u, on the threads set by orc_set_threads:
 * out[0] residual with local time steps, out[1] Jacobian assembly into a
 * zeroed matrix (the zeroing included), out[2] preconditioner setup of type
 * pctype (0 none, 1 point-block Jacobi, 2 SGS, 3 ILU(0)) in natural order,
 * out[3] one preconditioner apply.  The CPU-baseline timings of the bench. */
int orc_time_kernels(const void *h, const double *u, int pctype, int reps, double *out)
{
	const Disc *d = (const Disc *)h;
	if (reps < 1 || pctype < 0 || pctype > 3) return 1;
	const size_t n = (size_t)d->nelem();
	using clk = std::chrono::steady_clock;
	std::vector<double> t(reps + 1);
	auto timed = [&](auto &&fn) {
		for (int k = 0; k <= reps; k++) {
			const auto a = clk::now();
			if (int e = fn()) return e;
			t[k] = std::chrono::duration<double>(clk::now() - a).count();
		}
		std::sort(t.begin() + 1, t.end());
		return 0;
	};
	std::vector<double> r(4 * n), dt(n), z(4 * n);
	Disc::Work w;
	int e = timed([&] {
		std::fill(r.begin(), r.end(), 0.0);
		d->residual(u, r.data(), true, dt.data(), w);
		return 0;
	});
	if (e) return e;
	out[0] = t[1 + reps / 2];
	BSR A;
	A.setup(*d->m);
	if ((e = timed([&] {
		     std::fill(A.val.begin(), A.val.end(), 0.0);
		     return assemble_jacobian(*d, u, A);
	     })))
		return e;
	out[1] = t[1 + reps / 2];
	Precond pc;
	if ((e = timed([&] { return pc.setup(A, pctype, nullptr); }))) return e;
	out[2] = t[1 + reps / 2];
	if ((e = timed([&] {
		     pc.apply(r.data(), z.data());
		     return 0;
	     })))
		return e;
	out[3] = t[1 + reps / 2];
	return 0;
}

/* z = M^{-1} r for a BAIJ matrix given in (rowptr, col, val) form, with the
 * elimination order `order` (NULL = natural). */
int orc_precond_apply(int n, const int *rowptr, const int *col, const double *val, int type, const int *order,
                      const double *r, double *z)
{
	BSR A;
	A.n = n;
	A.rowptr.assign(rowptr, rowptr + n + 1);
	A.col.assign(col, col + rowptr[n]);
	A.val.assign(val, val + 16 * (size_t)rowptr[n]);
	A.diag.assign(n, -1);
	for (int i = 0; i < n; i++) A.diag[i] = A.find(i, i);
	Precond pc;
	if (int e = pc.setup(A, type, order)) return e;
	pc.apply(r, z);
	return 0;
}

/* FGMRES on a BAIJ system (x0 = 0); returns iterations; rnorm = final residual estimate */
int orc_fgmres(int n, const int *rowptr, const int *col, const double *val, int pctype, const int *order,
               const double *b, double *x, int restart, int maxit, double rtol, double *rnorm)
{
	BSR A;
	A.n = n;
	A.rowptr.assign(rowptr, rowptr + n + 1);
	A.col.assign(col, col + rowptr[n]);
	A.val.assign(val, val + 16 * (size_t)rowptr[n]);
	A.diag.assign(n, -1);
	for (int i = 0; i < n; i++) A.diag[i] = A.find(i, i);
	Precond pc;
	if (int e = pc.setup(A, pctype, order)) return -e;
	auto op = [&](const double *xx, double *y) { A.matvec(xx, y); };
	return fgmres(op, pc, b, x, 4 * (size_t)n, restart, maxit, rtol, rnorm);
}

/* cfg_d: cflmin, cflmax, tol, lin_rtol, mf_eps, min_relax
 * cfg_i: maxiter, abs_tol, pc, restart, lin_maxit, matrix_free, nl_update
 * stats_out: steps, lin_iters, status, res0, res, cfl (as doubles) */
int orc_steady_solve(const void *h, const double *cfg_d, const int *cfg_i, const int *pc_order, double *u,
                     double *stats_out, double *history)
{
	const Disc *d = (const Disc *)h;
	SolverCfg c;
	c.cflmin = cfg_d[0]; c.cflmax = cfg_d[1]; c.tol = cfg_d[2]; c.lin_rtol = cfg_d[3]; c.mf_eps = cfg_d[4];
	c.min_relax = cfg_d[5];
	c.maxiter = cfg_i[0]; c.abs_tol = cfg_i[1]; c.pc = cfg_i[2]; c.restart = cfg_i[3]; c.lin_maxit = cfg_i[4];
	c.matrix_free = cfg_i[5]; c.nl_update = cfg_i[6];
	SolveStats st;
	const int e = steady_solve(*d, c, u, st, pc_order, history);
	stats_out[0] = st.steps; stats_out[1] = st.lin_iters; stats_out[2] = st.status;
	stats_out[3] = st.res0; stats_out[4] = st.res; stats_out[5] = st.cfl;
	return e;
}

/* SteadyForwardEulerSolver::solve, aodesolver.cpp:136-282: u += cflinit dt/A r
 * with r = -R(u) and dt the local time steps; the ramped CFL the reference
 * computes is not used by its update.  The loop runs while the (relative, or
 * here optionally absolute) energy-residual norm exceeds tol; reaching
 * maxiter is a tolerance failure even on a converged last step, as there.
 * cfg_d: cflinit, tol; cfg_i: maxiter, abs_tol.  stats_out: steps, status, res0, res */
int orc_steady_fe(const void *h, const double *cfg_d, const int *cfg_i, double *u, double *stats_out, double *history)
{
	const Disc *d = (const Disc *)h;
	const Mesh &M = *d->m;
	const int ne = M.nelem;
	const double cflinit = cfg_d[0], tol = cfg_d[1];
	const int maxiter = cfg_i[0], abs_tol = cfg_i[1];
	std::vector<double> r(4 * (size_t)ne), dtm(ne);
	Disc::Work w;
	double resi = 1.0, initres = 1.0, res0 = 0;
	int step = 0, status = 0;
	while ((abs_tol ? resi > tol : resi / initres > tol) && step < maxiter) {
		std::fill(r.begin(), r.end(), 0.0);
		d->residual(u, r.data(), true, dtm.data(), w);
		for (int i = 0; i < ne; i++)
			for (int q = 0; q < 4; q++) u[4 * i + q] += cflinit * dtm[i] * 1.0 / M.area[i] * r[4 * i + q];
		double s = 0;
		for (int i = 0; i < ne; i++) s += r[4 * i + 3] * r[4 * i + 3] * M.area[i];
		resi = std::sqrt(s);
		if (step == 0) { initres = resi; res0 = resi; }
		if (history) history[step] = resi;
		step++;
		if (!std::isfinite(resi)) { status = 3; break; }
	}
	if (status == 0 && step == maxiter) status = 4;
	stats_out[0] = step; stats_out[1] = status; stats_out[2] = res0; stats_out[3] = resi;
	return status;
}

/* TVDRKSolver::solve, aodesolver.cpp:671-765 with initialize_TVDRK_Coeffs
 * (:45-67), as the reference has it: every stage evaluates the residual of
 * the step's starting state u (not of the stage state), the time step is
 * dtmin = min_i dt_i of the first stage, and a stage sets
 *   ustage = c0 u + c1 ustage - c2 dtmin cfl / A r,   r = -R(u),
 * until the elapsed time exceeds final_time - 1e-12 (A_SMALL_NUMBER).
 * out: steps, status (0, or 3 when dtmin is not finite), time */
int orc_tvdrk(const void *h, int order, double cfl, double final_time, double *u, double *out3)
{
	const Disc *d = (const Disc *)h;
	const Mesh &M = *d->m;
	const int ne = M.nelem;
	double co[3][3] = {{1, 0, 1}, {0, 0, 0}, {0, 0, 0}};
	if (order == 2) { co[1][0] = 0.5; co[1][1] = 0.5; co[1][2] = 0.5; }
	else if (order == 3) {
		co[1][0] = 0.75; co[1][1] = 0.25; co[1][2] = 0.25;
		co[2][0] = 0.3333333333333333; co[2][1] = 0.6666666666666667; co[2][2] = 0.6666666666666667;
	} else if (order != 1) return 1;
	std::vector<double> r(4 * (size_t)ne), dtm(ne), us(u, u + 4 * (size_t)ne);
	Disc::Work w;
	double time = 0;
	int step = 0, status = 0;
	while (time <= final_time - 1e-12) {
		double dtmin = 0;
		for (int s = 0; s < order; s++) {
			std::fill(r.begin(), r.end(), 0.0);
			d->residual(u, r.data(), true, dtm.data(), w);
			if (s == 0) dtmin = *std::min_element(dtm.begin(), dtm.end());
			if (!std::isfinite(dtmin)) { status = 3; break; }
			for (int i = 0; i < ne; i++)
				for (int q = 0; q < 4; q++)
					us[4 * i + q] = co[s][0] * u[4 * i + q] + co[s][1] * us[4 * i + q] -
					                co[s][2] * dtmin * cfl / M.area[i] * r[4 * i + q];
		}
		if (status) break;
		for (size_t k = 0; k < us.size(); k++) u[k] = us[k];
		step++;
		time += dtmin * cfl;
	}
	out3[0] = step; out3[1] = status; out3[2] = time;
	return status;
}

/* FlowFV_base::computeSurfaceData, flow_spatial.cpp:130-310: returns Cl, CDp, CDsf,
 * and (rows != NULL) the per-face output x, y, Cp, Cf of the marker's faces
 * (flow_spatial.cpp:168-237); returns the face count */
int orc_surface_data(const void *h, const double *u, int marker, double *out3, double *rows)
{
	const Disc *d = (const Disc *)h;
	const Mesh &M = *d->m;
	std::vector<double> grad(8 * (size_t)M.nelem);
	d->conserved_gradients(u, grad.data());
	const double wind[2] = {std::cos(d->aoa) * std::cos(0.0), std::sin(d->aoa) * std::cos(0.0)};
	const double pinf = 1.0 / (d->P.g * d->P.Minf * d->P.Minf);
	const double fnorm[2] = {-wind[1], wind[0]};
	double Cl = 0, Cdp = 0, Cdf = 0, tot = 0;
	int nrow = 0;
	for (int f = 0; f < M.nbface; f++) {
		if (M.btag[f] != marker) continue;
		const int le = M.intfac[4 * f];
		const double *n = &M.facemetric[3 * f];
		const double ar = n[2];
		const double tg[2] = {n[1], -n[0]};
		const double *ur = &u[4 * le];
		const double cp = (pressure_from_cons(d->P, ur) - pinf) * 2.0;
		const double mu = sutherland(d->P, temperature(d->P, ur[0], pressure_from_cons(d->P, ur)));
		const double *g = &grad[8 * le];
		double gu[2][2];
		for (int i = 0; i < 2; i++)
			for (int j = 0; j < 2; j++) gu[i][j] = (g[2 * (i + 1) + j] * ur[0] - ur[i + 1] * g[2 * 0 + j]) / (ur[0] * ur[0]);
		double force[2];
		for (int i = 0; i < 2; i++) {
			force[i] = 0;
			for (int j = 0; j < 2; j++) force[i] += (gu[i][j] + gu[j][i]) * n[j];
		}
		const double tauw = mu * (force[0] * tg[0] + force[1] * tg[1]);
		const double cf = 2 * tauw;
		const double ndotw = n[0] * wind[0] + n[1] * wind[1];
		const double ndotnw = n[0] * fnorm[0] + n[1] * fnorm[1];
		const double tdotw = tg[0] * wind[0] + tg[1] * wind[1];
		if (rows) {
			const int p0 = M.intfac[4 * f + 2], p1 = M.intfac[4 * f + 3];
			double *r = rows + 4 * (size_t)nrow;
			r[0] = (M.coords[2 * p0] + M.coords[2 * p1]) / 2;
			r[1] = (M.coords[2 * p0 + 1] + M.coords[2 * p1 + 1]) / 2;
			r[2] = cp;
			r[3] = cf;
		}
		nrow++;
		tot += ar;
		Cl += cp * ndotnw * ar;
		Cdp += cp * ndotw * ar;
		Cdf += cf * tdotw * ar;
	}
	out3[0] = Cl / tot; out3[1] = Cdp / tot; out3[2] = Cdf / tot;
	return nrow;
}

/* FlowOutput::compute_entropy_cell, aoutput.cpp:28-62 */
double orc_entropy_error(const void *h, const double *u)
{
	const Disc *d = (const Disc *)h;
	const Mesh &M = *d->m;
	auto ent = [&](const double *uc) { return pressure_from_cons(d->P, uc) / std::pow(uc[0], d->P.g); };
	const double sinf = ent(d->uinf);
	double err = 0;
	for (int i = 0; i < M.nelem; i++) {
		const double s = (ent(&u[4 * i]) - sinf) / sinf;
		err += s * s * M.area[i];
	}
	return std::sqrt(err);
}

// ---- pointwise entry points (restated physics; compared against the reference) ----
static Phys mkphys(const double *p)
{
	Phys P;
	P.g = p[0]; P.Minf = p[1]; P.Tinf = p[2]; P.Reinf = p[3]; P.Pr = p[4];
	return P;
}
int orc_flux(int kind, const double *phys, const double *ul, const double *ur, const double *n, double *f)
{
	return numerical_flux(kind, mkphys(phys), ul, ur, n, f);
}
int orc_flux_jacobian(int kind, const double *phys, const double *ul, const double *ur, const double *n, double *dfdl,
                      double *dfdr)
{
	if (kind == F_VANLEER || kind == F_AUSMPLUS) return 2;
	typedef Dual<8> D8;
	D8 a[4], b[4], F[4];
	for (int i = 0; i < 4; i++) {
		a[i] = D8(ul[i]); a[i].d[i] = 1;
		b[i] = D8(ur[i]); b[i].d[4 + i] = 1;
	}
	if (numerical_flux(kind, mkphys(phys), a, b, n, F)) return 1;
	for (int i = 0; i < 4; i++)
		for (int k = 0; k < 4; k++) { dfdl[4 * i + k] = -F[i].d[k]; dfdr[4 * i + k] = F[i].d[4 + k]; }
	return 0;
}
int orc_bc_ghost(int type, const double *phys, double aoa, const double *vals, const double *ins, const double *n,
                 double *gs)
{
	const Phys P = mkphys(phys);
	double uinf[4];
	freestream_state(P, aoa, uinf);
	BCSpec s; s.type = type; s.vals[0] = vals[0]; s.vals[1] = vals[1];
	return ghost_state(P, s, uinf, ins, n, gs);
}
int orc_bc_ghost_jacobian(int type, const double *phys, double aoa, const double *vals, const double *ins,
                          const double *n, double *gs, double *dgs)
{
	const Phys P = mkphys(phys);
	double uinf[4];
	freestream_state(P, aoa, uinf);
	BCSpec s; s.type = type; s.vals[0] = vals[0]; s.vals[1] = vals[1];
	return ghost_jacobian(P, s, uinf, ins, n, gs, dgs);
}
/* viscous flux from a prim-2 face gradient (NDIM x NVARS row-major) */
int orc_viscous_flux(int constvisc, const double *phys, const double *n, const double *grad, const double *ul,
                     const double *ur, double *vf)
{
	double g[2][4];
	std::memcpy(g, grad, sizeof(g));
	viscous_flux(mkphys(phys), constvisc != 0, n, g, ul, ur, vf);
	return 0;
}
/* thin-layer viscous flux Jacobian blocks: dvfi = -dF/dul, dvfj = dF/dur */
int orc_viscous_jacobian(int constvisc, const double *phys, const double *n, const double *rcl, const double *rcr,
                         const double *ul, const double *ur, double *dvfi, double *dvfj)
{
	typedef Dual<8> D8;
	D8 a[4], b[4], F[4];
	for (int i = 0; i < 4; i++) {
		a[i] = D8(ul[i]); a[i].d[i] = 1;
		b[i] = D8(ur[i]); b[i].d[4 + i] = 1;
	}
	viscous_flux_thinlayer(mkphys(phys), constvisc != 0, n, rcl, rcr, a, b, F);
	for (int i = 0; i < 4; i++)
		for (int k = 0; k < 4; k++) { dvfi[4 * i + k] = -F[i].d[k]; dvfj[4 * i + k] = F[i].d[4 + k]; }
	return 0;
}

}  // extern "C"
