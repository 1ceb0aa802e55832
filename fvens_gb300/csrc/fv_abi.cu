// C ABI of the GB300 hot path: mesh and discretisation handles, residual,
// gradients, Jacobian assembly and pointwise validation entry points.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <string>
#include <vector>

#include "../../include/fvens_gb300.h"
#include "fv_core.cuh"
#include "fv_abi_internal.hpp"
#include "fv_setup.hpp"

using namespace fvg;


namespace fvg {

static thread_local std::string g_last_error;
static std::atomic<long long> g_launches{0};

void set_error(const std::string &s) { g_last_error = s; }
void count_launches(long long n) { g_launches += n; }

fv_status cuda_status(cudaError_t e, const char *what)
{
	if (e == cudaSuccess) return FV_OK;
	set_error(std::string(what) + ": " + cudaGetErrorString(e));
	return FV_ERR_CUDA;
}

template <class T>
static cudaError_t dalloc(T **p, size_t n, std::vector<void *> *owned)
{
	*p = nullptr;
	if (n == 0) n = 1;
	cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
	if (e == cudaSuccess && owned) owned->push_back((void *)*p);
	return e;
}

template <class T>
static cudaError_t dupload(T **p, const std::vector<T> &h, std::vector<void *> *owned)
{
	cudaError_t e = dalloc(p, h.size(), owned);
	if (e != cudaSuccess) return e;
	if (!h.empty()) e = cudaMemcpy(*p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
	return e;
}

/* Uploads the mesh arrays the kernels read (see the layout notes in fv_core.cuh). */
static fv_status mesh_upload(fv_mesh_impl *m)
{
	if (m->dev_ready) return FV_OK;
	const HostMesh &h = m->h;
	DevMesh &d = m->d;
	d.nelem = h.nelem; d.nbface = h.nbface; d.naface = h.naface; d.ncolors = h.ncolors;
	const MeshArrays a = mesh_arrays(h);
	const std::vector<double2> &cc = a.cc, &fcen = a.fcen, &gcen = a.gcen;
	const std::vector<double> &area = a.area, &iarea = a.iarea;
	const std::vector<int4> &cface = a.cface, &cnbr = a.cnbr, &crev = a.crev;
	const std::vector<int2> &flr = a.flr, &fslot = a.fslot;
	const std::vector<d4> &fgeo = a.fgeo;
	cudaError_t e = cudaSuccess;
	std::vector<void *> *own = nullptr;
	if (!e) e = dupload(&d.cc, cc, own);
	if (!e) e = dupload(&d.area, area, own);
	if (!e) e = dupload(&d.iarea, iarea, own);
	if (!e) e = dupload(&d.cface, cface, own);
	if (!e) e = dupload(&d.cnbr, cnbr, own);
	if (!e) e = dupload(&d.cslot_rev, crev, own);
	if (!e) e = dupload(&d.flr, flr, own);
	if (!e) e = dupload(&d.fslot, fslot, own);
	if (!e) e = dupload(&d.fgeo, fgeo, own);
	if (!e) e = dupload(&d.fcen, fcen, own);
	if (!e) e = dupload(&d.gcen, gcen, own);
	if (!e) e = dupload(&d.color_cells, h.color_cells, own);
	d.color_ptr = h.color_ptr;
	if (e) return cuda_status(e, "mesh upload");
	m->dev_ready = true;
	return FV_OK;
}

static void mesh_free(fv_mesh_impl *m)
{
	DevMesh &d = m->d;
	void *ps[] = {d.cc, d.area, d.iarea, d.cface, d.cnbr, d.cslot_rev, d.flr, d.fslot, d.fgeo, d.fcen, d.gcen, d.color_cells};
	for (void *p : ps)
		if (p) cudaFree(p);
	m->dev_ready = false;
}

Phys make_phys(const fv_physics_cfg &c)
{
	Phys P;
	std::memset(&P, 0, sizeof(P));
	P.g = c.gamma; P.gm1 = c.gamma - 1.0; P.igm1 = 1.0 / (c.gamma - 1.0);
	P.Minf = c.Minf; P.Tinf = c.Tinf; P.Reinf = c.Reinf; P.Pr = c.Pr;
	P.tcoef = c.gamma * c.Minf * c.Minf;
	P.pinf = 1.0 / (c.gamma * c.Minf * c.Minf);
	P.sutC = 110.5 / c.Tinf;
	P.sutK = (1.0 + P.sutC) / c.Reinf;
	P.kcoef = 1.0 / (c.Minf * c.Minf * (c.gamma - 1.0) * c.Pr);
	P.ivisc = 1.0 / c.Reinf;
	P.aoa = c.aoa;
	P.uinf[0] = 1.0;
	P.uinf[1] = std::cos(c.aoa) * std::cos(0.0);
	P.uinf[2] = std::sin(c.aoa) * std::cos(0.0);
	P.uinf[3] = P.pinf / (c.gamma - 1.0) + 0.5 * 1.0 * 1.0;
	P.pinf_cons = (c.gamma - 1.0) * (P.uinf[3] - 0.5 * (P.uinf[1] * P.uinf[1] + P.uinf[2] * P.uinf[2]) / P.uinf[0]);
	return P;
}

}  // namespace fvg

extern "C" {

int fv_abi_version(void) { return FVENS_GB300_ABI_VERSION; }

const char *fv_status_string(fv_status s)
{
	switch (s) {
	case FV_OK: return "ok";
	case FV_ERR_INVALID: return "invalid argument";
	case FV_ERR_CUDA: return "CUDA error";
	case FV_ERR_NUMERICAL: return "numerical error: residual is NaN or inf";
	case FV_ERR_TOLERANCE: return "did not converge to the specified tolerance";
	case FV_ERR_UNSUPPORTED: return "not implemented by the reference discretisation";
	case FV_ERR_MESH: return "mesh error";
	}
	return "unknown status";
}

const char *fv_last_error(void) { return g_last_error.c_str(); }
long long fv_kernel_launch_count(void) { return g_launches.load(); }

static fv_status finish_mesh(fv_mesh *m, int rc, const std::string &err, fv_mesh **out)
{
	if (rc) {
		set_error(err);
		delete m;
		return FV_ERR_MESH;
	}
	*out = m;
	return FV_OK;
}

fv_status fv_mesh_create(const fv_mesh_desc *desc, int reorder, fv_mesh **out)
{
	if (!desc || !out) { set_error("null argument"); return FV_ERR_INVALID; }
	fv_mesh *m = new fv_mesh();
	std::string err;
	const int rc = mesh_from_arrays(m->h, desc->npoin, desc->coords, desc->nelem, desc->nnode, desc->inpoel,
	                                desc->nbface, desc->bface, desc->btag, reorder, &err);
	return finish_mesh(m, rc, err, out);
}

fv_status fv_mesh_generate(int kind, const double *p, int np, int reorder, fv_mesh **out)
{
	if (!out || !p) { set_error("null argument"); return FV_ERR_INVALID; }
	RawMesh r;
	if (kind == FV_MESH_CHANNEL_BUMP && np >= 4) {
		r = gen_channel_bump((int)p[0], (int)p[1], p[2], (uint64_t)p[3]);
	} else if (kind == FV_MESH_NACA_OGRID && np >= 8) {
		r = gen_naca_ogrid((int)p[0], (int)p[1], p[2], (int)p[3], p[4], p[5], (int)p[6], (uint64_t)p[7]);
	} else if (kind == FV_MESH_NACA_HYBRID && np >= 6) {
		if (p[0] < 8 || p[1] < 0 || p[2] <= 0 || p[3] < 1 || p[4] <= 1 || p[5] < 0 || p[5] > 1) {
			set_error("invalid hybrid NACA mesh parameters");
			return FV_ERR_INVALID;
		}
		r = gen_naca_hybrid((int)p[0], (int)p[1], p[2], p[3], p[4], p[5]);
	} else {
		set_error("unknown mesh kind or too few parameters");
		return FV_ERR_INVALID;
	}
	fv_mesh *m = new fv_mesh();
	std::string err;
	const int rc = mesh_from_arrays(m->h, r.npoin, r.coords.data(), r.nelem, r.nnode.data(), r.inpoel.data(), r.nbface,
	                                r.bface.data(), r.btag.data(), reorder, &err);
	return finish_mesh(m, rc, err, out);
}

fv_status fv_mesh_read_gmsh(const char *path, int reorder, fv_mesh **out)
{
	if (!path || !out) { set_error("null argument"); return FV_ERR_INVALID; }
	RawMesh r;
	std::string err;
	if (read_gmsh2(path, r, &err)) { set_error(err); return FV_ERR_MESH; }
	fv_mesh *m = new fv_mesh();
	const int rc = mesh_from_arrays(m->h, r.npoin, r.coords.data(), r.nelem, r.nnode.data(), r.inpoel.data(), r.nbface,
	                                r.bface.data(), r.btag.data(), reorder, &err);
	return finish_mesh(m, rc, err, out);
}

fv_status fv_mesh_read_su2(const char *path, int reorder, fv_mesh **out)
{
	if (!path || !out) { set_error("null argument"); return FV_ERR_INVALID; }
	RawMesh r;
	std::string err;
	if (read_su2(path, r, &err)) { set_error(err); return FV_ERR_MESH; }
	fv_mesh *m = new fv_mesh();
	const int rc = mesh_from_arrays(m->h, r.npoin, r.coords.data(), r.nelem, r.nnode.data(), r.inpoel.data(), r.nbface,
	                                r.bface.data(), r.btag.data(), reorder, &err);
	return finish_mesh(m, rc, err, out);
}

/* readMesh (meshreaders.cpp:33-50): the format from the file extension */
fv_status fv_mesh_read(const char *path, int reorder, fv_mesh **out)
{
	if (!path || !out) { set_error("null argument"); return FV_ERR_INVALID; }
	const std::string p(path);
	const size_t dot = p.rfind('.');
	const std::string ext = dot == std::string::npos ? "" : p.substr(dot + 1);
	if (ext == "msh") return fv_mesh_read_gmsh(path, reorder, out);
	if (ext == "su2") return fv_mesh_read_su2(path, reorder, out);
	set_error("unknown mesh file extension: " + ext);
	return FV_ERR_INVALID;
}

fv_status fv_mesh_find_lines(fv_mesh *m, double threshold, int *nlines, int *cell_line)
{
	if (!m) { set_error("null argument"); return FV_ERR_INVALID; }
	const int nl = threshold > 0 ? find_lines(m->h, threshold) : 0;
	if (threshold <= 0) {
		m->h.lines.clear();
		m->h.cell_line.assign(m->h.nelem, -1);
	}
	if (nlines) *nlines = nl;
	if (cell_line) std::copy(m->h.cell_line.begin(), m->h.cell_line.end(), cell_line);
	return FV_OK;
}

}  // extern "C"

namespace {

/* SPARSEPACK GENRCM (A. George and J. W. Liu, Computer Solution of Large
 * Sparse Positive Definite Systems, 1981), the ordering behind PETSc's
 * MatGetOrdering "rcm": per connected component, in order of the lowest
 * unnumbered vertex, a pseudo-peripheral root (FNROOT: restart from a vertex
 * of minimum degree in the last level while the level structure deepens),
 * then breadth-first numbering with each vertex's new neighbours in
 * increasing degree (stable), reversed.  adj: sorted neighbour lists without
 * the vertex itself.  Returns the vertex at each position. */
std::vector<int> genrcm(const std::vector<std::vector<int>> &adj)
{
	const int n = (int)adj.size();
	std::vector<char> mask(n, 1), seen(n, 0);
	std::vector<int> out, deg(n), ls, lp;
	out.reserve(n);
	auto rootls = [&](int root) {  // level structure of root's unnumbered component
		ls.assign(1, root);
		lp.assign(1, 0);
		seen[root] = 1;
		size_t b = 0;
		while (true) {
			const size_t e = ls.size();
			for (size_t i = b; i < e; i++)
				for (int x : adj[ls[i]])
					if (mask[x] && !seen[x]) { seen[x] = 1; ls.push_back(x); }
			if (ls.size() == e) break;
			lp.push_back((int)e);
			b = e;
		}
		for (int x : ls) seen[x] = 0;
	};
	auto degree = [&](int v) { int d = 0; for (int x : adj[v]) d += mask[x]; return d; };
	for (int s = 0; s < n; s++) {
		if (!mask[s]) continue;
		int root = s;
		rootls(root);
		int nlvl = (int)lp.size();
		const int ccsize = (int)ls.size();
		while (nlvl > 1 && nlvl < ccsize) {
			const int j0 = lp.back();
			int mindeg = ccsize;
			root = ls[j0];
			if (ccsize - j0 > 1)
				for (int j = j0; j < ccsize; j++) {
					const int d = degree(ls[j]);
					if (d < mindeg) { root = ls[j]; mindeg = d; }
				}
			rootls(root);
			if ((int)lp.size() <= nlvl) break;
			nlvl = (int)lp.size();
		}
		for (int x : ls) deg[x] = degree(x);
		const size_t c0 = out.size();
		out.push_back(root);
		mask[root] = 0;
		for (size_t i = c0; i < out.size(); i++) {
			const size_t f = out.size();
			for (int x : adj[out[i]])
				if (mask[x]) { mask[x] = 0; out.push_back(x); }
			std::stable_sort(out.begin() + f, out.end(), [&](int a, int b) { return deg[a] < deg[b]; });
		}
		std::reverse(out.begin() + c0, out.end());
	}
	return out;
}

}  // namespace

extern "C" {

/* getHybridLineOrdering (meshordering.cpp:69-141, 267-402): a graph whose
 * vertices are the lines, then the cells outside lines; two vertices are
 * adjacent when a cell of one shares a face with a cell of the other.  The
 * graph is taken in natural order or reordered by RCM, and each line vertex
 * expands to its cells in line order. */
fv_status fv_mesh_line_ordering(const fv_mesh *m, int rcm, int *order)
{
	if (!m || !order) { set_error("null argument"); return FV_ERR_INVALID; }
	const HostMesh &h = m->h;
	const int nl = (int)h.lines.size();
	std::vector<int> points, vid(h.nelem);
	for (int c = 0; c < h.nelem; c++) {
		if (!h.cell_line.empty() && h.cell_line[c] >= 0) {
			vid[c] = h.cell_line[c];
		} else {
			vid[c] = nl + (int)points.size();
			points.push_back(c);
		}
	}
	const int nv = nl + (int)points.size();
	std::vector<int> gorder(nv);
	for (int v = 0; v < nv; v++) gorder[v] = v;
	if (rcm) {
		std::vector<std::vector<int>> adj(nv);
		for (int f = h.nbface; f < h.naface; f++) {
			const int a = vid[h.face_l[f]], b = vid[h.face_r[f]];
			if (a != b) { adj[a].push_back(b); adj[b].push_back(a); }
		}
		for (std::vector<int> &a : adj) {
			std::sort(a.begin(), a.end());
			a.erase(std::unique(a.begin(), a.end()), a.end());
		}
		gorder = genrcm(adj);
	}
	int k = 0;
	for (int v : gorder) {
		if (v < nl)
			for (int c : h.lines[v]) order[k++] = c;
		else
			order[k++] = points[v - nl];
	}
	if (k != h.nelem) { set_error("inconsistent lines"); return FV_ERR_MESH; }
	return FV_OK;
}

fv_status fv_mesh_periodic_map(const fv_mesh *m, int marker, int axis, int *map)
{
	if (!m || !map) { set_error("null argument"); return FV_ERR_INVALID; }
	if (axis < 0 || axis > 1) { set_error("periodic axis must be 0 or 1"); return FV_ERR_INVALID; }
	const std::vector<int> pm = periodic_map(m->h, marker, axis);
	std::copy(pm.begin(), pm.end(), map);
	return FV_OK;
}

fv_status fv_mesh_counts(const fv_mesh *m, int c[6])
{
	if (!m || !c) { set_error("null argument"); return FV_ERR_INVALID; }
	c[0] = m->h.nelem; c[1] = m->h.nbface; c[2] = m->h.ninface; c[3] = m->h.naface; c[4] = m->h.npoin;
	c[5] = m->h.ncolors;
	return FV_OK;
}

fv_status fv_mesh_export(const fv_mesh *m, double *coords, int *nnode, int *inpoel, int *bface, int *btag, int *perm)
{
	if (!m) { set_error("null argument"); return FV_ERR_INVALID; }
	const HostMesh &h = m->h;
	if (coords) std::memcpy(coords, h.coords.data(), sizeof(double) * h.coords.size());
	if (nnode) std::memcpy(nnode, h.nnode.data(), sizeof(int) * h.nnode.size());
	if (inpoel) std::memcpy(inpoel, h.inpoel.data(), sizeof(int) * h.inpoel.size());
	if (bface) std::memcpy(bface, h.bface.data(), sizeof(int) * h.bface.size());
	if (btag) std::memcpy(btag, h.btag.data(), sizeof(int) * h.btag.size());
	if (perm) std::memcpy(perm, h.perm.data(), sizeof(int) * h.perm.size());
	return FV_OK;
}

fv_status fv_mesh_geometry(const fv_mesh *m, int *face_lr, double *fnorm, double *area, double *cc, int *color)
{
	if (!m) { set_error("null argument"); return FV_ERR_INVALID; }
	const HostMesh &h = m->h;
	if (face_lr)
		for (int f = 0; f < h.naface; f++) { face_lr[2 * f] = h.face_l[f]; face_lr[2 * f + 1] = h.face_r[f]; }
	if (fnorm) std::memcpy(fnorm, h.fnorm.data(), sizeof(double) * h.fnorm.size());
	if (area) std::memcpy(area, h.area.data(), sizeof(double) * h.area.size());
	if (cc) std::memcpy(cc, h.cc.data(), sizeof(double) * h.cc.size());
	if (color) std::memcpy(color, h.color.data(), sizeof(int) * h.color.size());
	return FV_OK;
}

void fv_mesh_destroy(fv_mesh *m)
{
	if (!m) return;
	mesh_free(m);
	delete m;
}

fv_status fv_disc_create(fv_mesh *m, const fv_physics_cfg *phys, int batch, const fv_numerics_cfg *num,
                         const fv_bc_cfg *bcs, int nbc, fv_disc **out)
{
	if (!m || !phys || !num || (nbc > 0 && !bcs) || !out || batch < 1) {
		set_error("null argument or batch < 1");
		return FV_ERR_INVALID;
	}
	if (num->conv_numflux < 0 || num->conv_numflux > 6 || num->conv_numflux_jac < 0 || num->conv_numflux_jac > 6 ||
	    num->gradientscheme < 0 || num->gradientscheme > 2 || num->reconstruction < 0 || num->reconstruction > 4) {
		set_error("unknown flux, gradient or reconstruction scheme");
		return FV_ERR_INVALID;
	}
	const HostMesh &h = m->h;
	fv_disc *D = new fv_disc();
	D->mesh = m;
	D->batch = batch;
	cudaGetDevice(&D->device);
	// BC table (create_const_flowBCs, abc.cpp:460-500)
	std::map<int, int> tag2idx;
	for (int k = 0; k < nbc; k++) {
		const int t = bcs[k].bc_type;
		if (t < 0 || t > 7 || t == FV_BC_PERIODIC) {
			set_error("BC type not implemented yet!");
			delete D;
			return FV_ERR_UNSUPPORTED;
		}
		tag2idx[bcs[k].bc_tag] = (int)D->bcs_h.size();
		D->bcs_h.push_back(BCDev{t, bcs[k].bc_vals[0], bcs[k].bc_vals[1]});
	}
	std::vector<int> bcid(std::max(h.nbface, 1), 0);
	for (int f = 0; f < h.nbface; f++) {
		auto it = tag2idx.find(h.btag[f]);
		if (it == tag2idx.end()) {
			set_error("no boundary condition for boundary marker " + std::to_string(h.btag[f]));
			delete D;
			return FV_ERR_INVALID;
		}
		bcid[f] = it->second;
	}
	for (int b = 0; b < batch; b++) D->phys_h.push_back(make_phys(phys[b]));
	fv_status st = mesh_upload(m);
	if (st) { delete D; return st; }
	// per-face / per-cell precomputation
	const int ne = h.nelem, nf = h.naface, nb = h.nbface;
	const DiscArrays da = disc_arrays(h, num->reconstruction == FV_REC_VENKATAKRISHNAN, num->limiter_param);
	const bool ls = num->gradientscheme == FV_GRAD_LEASTSQUARES;
	const std::vector<d4> &gcoef = ls ? da.gcoef_ls : da.gcoef_gg;
	const std::vector<d4> &fvis = da.fvis;
	const std::vector<double> &veps2 = da.veps2;
	DiscDev &d = D->d;
	std::memset(&d, 0, sizeof(d));
	d.nelem = ne; d.nbface = nb; d.naface = nf; d.batch = batch;
	const DevMesh &dm = m->d;
	d.cc = dm.cc; d.area = dm.area; d.iarea = dm.iarea; d.cface = dm.cface; d.cnbr = dm.cnbr;
	d.flr = dm.flr; d.fgeo = dm.fgeo; d.fcen = dm.fcen; d.gcen = dm.gcen;
	d.flux = num->conv_numflux; d.jflux = num->conv_numflux_jac;
	d.gradscheme = num->order2 ? num->gradientscheme : FV_GRAD_NONE;
	d.recon = num->reconstruction;
	d.order2 = num->order2 && num->gradientscheme != FV_GRAD_NONE;
	d.viscous = phys[0].viscous_sim; d.constvisc = phys[0].const_visc;
	d.limparam = num->limiter_param;
	cudaError_t e = cudaSuccess;
	std::vector<void *> *own = &D->owned;
	int *bcid_d; BCDev *bcs_d; Phys *phys_d; d4 *gcoef_d, *fvis_d; double2 *gself_d; double *veps_d;
	if (!e) e = dupload(&bcid_d, bcid, own);
	if (!e) e = dupload(&bcs_d, D->bcs_h.empty() ? std::vector<BCDev>(1, BCDev{0, 0, 0}) : D->bcs_h, own);
	if (!e) e = dupload(&phys_d, D->phys_h, own);
	if (!e) e = dupload(&gcoef_d, gcoef, own);
	if (!e) e = dupload(&gself_d, da.gself_gg, own);
	if (!e) e = dupload(&fvis_d, fvis, own);
	if (!e) e = dupload(&veps_d, veps2, own);
	d.bcid = bcid_d; d.bcs = bcs_d; d.phys = phys_d; d.gcoef = gcoef_d; d.gself = gself_d; d.fvis = fvis_d;
	d.veps2 = veps_d;
	ResidualWork &w = D->w;
	const size_t B = batch;
	if (!e) e = dalloc(&w.prim, B * ne, own);
	if (!e) e = dalloc(&w.ghost_prim, B * std::max(nb, 1), own);
	if (!e) e = dalloc(&w.ghost_cons, B * std::max(nb, 1), own);
	if (!e) e = dalloc(&w.grad, 2 * B * ne, own);
	if (!e) e = dalloc(&w.lgrad, recon_gradients(num->reconstruction) ? 2 * B * ne : 1, own);
	if (!e) e = dalloc(&w.fflux, B * nf, own);
	if (!e) e = dalloc(&w.spec, B * nf, own);
	if (!e) e = dupload(&D->btag, nb > 0 ? h.btag : std::vector<int>(1, 0), own);
	if (!e) e = dalloc(&D->surf, 4 * B, own);
	if (e) {
		st = cuda_status(e, "discretisation setup");
		fv_disc_destroy(D);
		return st;
	}
	*out = D;
	return FV_OK;
}

void fv_disc_destroy(fv_disc *D)
{
	if (!D) return;
	for (void *p : D->owned) cudaFree(p);
	delete D;
}

fv_status fv_disc_set_stream(fv_disc *D, void *stream)
{
	if (!D) { set_error("null argument"); return FV_ERR_INVALID; }
	D->stream = (cudaStream_t)stream;
	return FV_OK;
}

fv_status fv_disc_synchronize(fv_disc *D)
{
	if (!D) { set_error("null argument"); return FV_ERR_INVALID; }
	return cuda_status(cudaStreamSynchronize(D->stream), "synchronize");
}

fv_status fv_disc_freestream(const fv_disc *D, double *u)
{
	if (!D || !u) { set_error("null argument"); return FV_ERR_INVALID; }
	for (int b = 0; b < D->batch; b++)
		for (int k = 0; k < 4; k++) u[4 * b + k] = D->phys_h[b].uinf[k];
	return FV_OK;
}

fv_status fv_compute_residual(fv_disc *D, const double *u, double *r, int gettimesteps, double *dt)
{
	if (!D || !u || !r || (gettimesteps && !dt)) { set_error("null argument"); return FV_ERR_INVALID; }
	const int before = D->kernels_launched;
	const cudaError_t e = residual_launch(D, u, r, gettimesteps, dt, D->stream);
	count_launches(D->kernels_launched - before);
	return cuda_status(e, "residual");
}

fv_status fv_disc_autotune(fv_disc *D, const double *u, int *h_block_sizes)
{
	if (!D || !u) { set_error("null argument"); return FV_ERR_INVALID; }
	const int before = D->kernels_launched;
	const cudaError_t e = residual_autotune(D, u, D->stream, h_block_sizes);
	count_launches(D->kernels_launched - before);
	return cuda_status(e, "autotune");
}

fv_status fv_disc_block_sizes(const fv_disc *D, int n, int *h_block_sizes)
{
	if (!D || !h_block_sizes || n < 1) { set_error("null argument or n < 1"); return FV_ERR_INVALID; }
	for (int k = 0; k < n && k < KBS_COUNT; k++) h_block_sizes[k] = D->bs[k];
	return FV_OK;
}

fv_status fv_get_gradients(fv_disc *D, const double *u, double *grad, int primitive)
{
	if (!D || !u || !grad) { set_error("null argument"); return FV_ERR_INVALID; }
	const int before = D->kernels_launched;
	const cudaError_t e = gradients_launch(D, u, grad, !primitive, D->stream);
	count_launches(D->kernels_launched - before);
	return cuda_status(e, "gradients");
}

fv_status fv_matrix_create(fv_disc *D, int precision, fv_matrix **out)
{
	if (!D || !out || (precision != 4 && precision != 8)) { set_error("invalid argument"); return FV_ERR_INVALID; }
	fv_matrix *M = new fv_matrix();
	M->owner = D;
	M->A.nelem = D->d.nelem;
	M->A.batch = D->batch;
	M->A.prec = precision;
	cudaError_t e = cudaMalloc(&M->A.val, M->A.nval() * precision);
	if (!e) e = cudaMemset(M->A.val, 0, M->A.nval() * precision);
	if (!e) e = cudaMalloc((void **)&M->A.bdiag, sizeof(double) * 16 * (size_t)D->batch * std::max(D->d.nbface, 1));
	if (e) {
		fv_matrix_destroy(M);
		return cuda_status(e, "matrix allocation");
	}
	*out = M;
	return FV_OK;
}

void fv_matrix_destroy(fv_matrix *M)
{
	if (!M) return;
	if (M->A.val) cudaFree(M->A.val);
	if (M->A.bdiag) cudaFree(M->A.bdiag);
	delete M;
}

fv_status fv_assemble_jacobian(fv_disc *D, const double *u, fv_matrix *M)
{
	if (!D || !u || !M || M->owner != D) { set_error("invalid argument"); return FV_ERR_INVALID; }
	if (D->d.jflux == FV_FLUX_VANLEER) {
		set_error(" ! VanLeerFlux: Not implemented!");
		return FV_ERR_UNSUPPORTED;
	}
	if (D->d.jflux == FV_FLUX_AUSMPLUS) {
		set_error(" ! AUSMPlusFlux: Not implemented!");
		return FV_ERR_UNSUPPORTED;
	}
	const int before = D->kernels_launched;
	const cudaError_t e = jacobian_launch(D, u, M->A, D->stream);
	count_launches(D->kernels_launched - before);
	return cuda_status(e, "jacobian assembly");
}

fv_status fv_matrix_add_diagonal(fv_disc *D, fv_matrix *M, const double *diag)
{
	if (!D || !M || !diag) { set_error("null argument"); return FV_ERR_INVALID; }
	const cudaError_t e = matrix_add_diag_launch(M->A, diag, D->stream);
	count_launches(1);
	return cuda_status(e, "matrix add diagonal");
}

fv_status fv_matrix_to_host(fv_disc *D, const fv_matrix *M, int member, int *nnzb, int *rowptr, int *col, double *val)
{
	if (!D || !M || !nnzb || member < 0 || member >= D->batch) { set_error("invalid argument"); return FV_ERR_INVALID; }
	const HostMesh &h = D->mesh->h;
	const int ne = h.nelem;
	int nz = ne;
	for (int i = 0; i < ne; i++)
		for (int j = 0; j < h.nnode[i]; j++)
			if (h.esuel[4 * i + j] >= 0) nz++;
	*nnzb = nz;
	if (!val) return FV_OK;
	const size_t per = (size_t)5 * ne * 16;
	std::vector<double> hv(per);
	cudaError_t e = cudaStreamSynchronize(D->stream);
	if (!e) {
		if (M->A.prec == 4) {
			std::vector<float> tmp(per);
			e = cudaMemcpy(tmp.data(), (const float *)M->A.val + member * per, per * 4, cudaMemcpyDeviceToHost);
			for (size_t k = 0; k < per; k++) hv[k] = tmp[k];
		} else {
			e = cudaMemcpy(hv.data(), (const double *)M->A.val + member * per, per * 8, cudaMemcpyDeviceToHost);
		}
	}
	if (e) return cuda_status(e, "matrix copy");
	int k = 0;
	rowptr[0] = 0;
	for (int i = 0; i < ne; i++) {
		std::vector<std::pair<int, int>> cs{{i, 0}};
		for (int j = 0; j < h.nnode[i]; j++)
			if (h.esuel[4 * i + j] >= 0) cs.push_back({h.esuel[4 * i + j], 1 + j});
		std::sort(cs.begin(), cs.end());
		for (auto &c : cs) {
			col[k] = c.first;
			std::memcpy(&val[16 * (size_t)k], &hv[((size_t)c.second * ne + i) * 16], 16 * sizeof(double));
			k++;
		}
		rowptr[i + 1] = k;
	}
	return FV_OK;
}

fv_status fv_pointwise_flux(fv_disc *D, int kind, int n, const double *ul, const double *ur, const double *nrm, double *f)
{
	if (!D || n < 0 || kind < 0 || kind > 6) { set_error("invalid argument"); return FV_ERR_INVALID; }
	const cudaError_t e = pointwise_flux_launch(D, kind, n, ul, ur, nrm, f, D->stream);
	count_launches(1);
	return cuda_status(e, "pointwise flux");
}

fv_status fv_pointwise_flux_jacobian(fv_disc *D, int kind, int n, const double *ul, const double *ur, const double *nrm,
                                     double *dfdl, double *dfdr)
{
	if (!D || n < 0 || kind < 0 || kind > 6) { set_error("invalid argument"); return FV_ERR_INVALID; }
	if (kind == FV_FLUX_VANLEER || kind == FV_FLUX_AUSMPLUS) {
		set_error("the reference implements no Jacobian for this flux");
		return FV_ERR_UNSUPPORTED;
	}
	const cudaError_t e = pointwise_flux_jac_launch(D, kind, n, ul, ur, nrm, dfdl, dfdr, D->stream);
	count_launches(1);
	return cuda_status(e, "pointwise flux jacobian");
}

fv_status fv_pointwise_bc(fv_disc *D, int bc_type, const double *vals, int n, const double *in, const double *nrm,
                          double *ghost, double *jac_ghost, double *dgdu)
{
	if (!D || !vals || n < 0 || bc_type < 0 || bc_type > 7 || bc_type == FV_BC_PERIODIC) {
		set_error("invalid argument");
		return FV_ERR_INVALID;
	}
	const cudaError_t e = pointwise_bc_launch(D, BCDev{bc_type, vals[0], vals[1]}, n, in, nrm, ghost, jac_ghost, dgdu,
	                                          D->stream);
	count_launches(1);
	return cuda_status(e, "pointwise bc");
}

}  // extern "C"

extern "C" fv_status fv_mesh_block_order(const fv_mesh *m, int part_size, int *order, int *nparts, int *ncolors)
{
	return fv_mesh_block_order_ex(m, part_size, 0, order, nparts, ncolors);
}

extern "C" fv_status fv_mesh_block_order_ex(const fv_mesh *m, int part_size, int colouring, int *order, int *nparts,
                                            int *ncolors)
{
	if (!m || !order || part_size < 1 || colouring < 0 || colouring > 1) {
		set_error("invalid argument");
		return FV_ERR_INVALID;
	}
	const BlockOrder bo = block_colour_order(m->h, part_size, colouring);
	std::memcpy(order, bo.pos_cell.data(), sizeof(int) * bo.pos_cell.size());
	if (nparts) *nparts = bo.nparts;
	if (ncolors) *ncolors = bo.ncolors;
	return FV_OK;
}
