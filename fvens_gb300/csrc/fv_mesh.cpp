// Host mesh construction for the GB300 hot path; see fv_mesh.hpp.
#include "fv_mesh.hpp"

#include <algorithm>
#include <set>
#include <tuple>
#include <array>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <limits>
#include <numeric>
#include <sstream>
#include <unordered_map>

namespace fvg {

namespace {

constexpr int kUnmatched = -2147483647;

uint64_t splitmix64(uint64_t &s)
{
	uint64_t z = (s += 0x9E3779B97F4A7C15ull);
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
	return z ^ (z >> 31);
}

inline uint64_t edge_key(int a, int b)
{
	const uint32_t lo = (uint32_t)std::min(a, b), hi = (uint32_t)std::max(a, b);
	return ((uint64_t)lo << 32) | hi;
}

double tri_area(const double *c, int a, int b, int d)
{
	const double xa = c[2 * a], ya = c[2 * a + 1], xb = c[2 * b], yb = c[2 * b + 1], xd = c[2 * d], yd = c[2 * d + 1];
	return 0.5 * (xa * (yb - yd) - ya * (xb - xd) + xb * yd - xd * yb);
}

double cell_area(const double *c, const int *e, int nn)
{
	double a = tri_area(c, e[0], e[1], e[2]);
	if (nn == 4) a += tri_area(c, e[0], e[2], e[3]);
	return a;
}

struct EdgeRef {
	uint64_t key;
	int cell, local;
};

// Sort all cell edges by node-pair key; returns the sorted list.
std::vector<EdgeRef> sorted_edges(int nelem, const std::vector<int> &nnode, const std::vector<int> &inpoel)
{
	std::vector<EdgeRef> e;
	e.reserve(4 * (size_t)nelem);
	for (int i = 0; i < nelem; i++)
		for (int j = 0; j < nnode[i]; j++)
			e.push_back({edge_key(inpoel[4 * i + j], inpoel[4 * i + (j + 1) % nnode[i]]), i, j});
	std::sort(e.begin(), e.end(), [](const EdgeRef &a, const EdgeRef &b) {
		return a.key < b.key || (a.key == b.key && (a.cell < b.cell || (a.cell == b.cell && a.local < b.local)));
	});
	return e;
}

}  // namespace

std::vector<int> rcm_order(int n, const std::vector<int> &ptr, const std::vector<int> &adj)
{
	std::vector<int> deg(n);
	for (int i = 0; i < n; i++) deg[i] = ptr[i + 1] - ptr[i];
	std::vector<int> order;
	order.reserve(n);
	std::vector<char> done(n, 0);
	std::vector<int> level(n, -1);
	auto bfs_levels = [&](int s, std::vector<int> &lastlev) {
		// returns eccentricity; fills lastlev with nodes at the deepest level
		std::vector<int> q{s};
		std::vector<int> seen;
		level[s] = 0;
		seen.push_back(s);
		size_t h = 0;
		int ecc = 0;
		while (h < q.size()) {
			const int v = q[h++];
			ecc = std::max(ecc, level[v]);
			for (int k = ptr[v]; k < ptr[v + 1]; k++) {
				const int w = adj[k];
				if (level[w] < 0 && !done[w]) {
					level[w] = level[v] + 1;
					q.push_back(w);
					seen.push_back(w);
				}
			}
		}
		lastlev.clear();
		for (int v : seen)
			if (level[v] == ecc) lastlev.push_back(v);
		for (int v : seen) level[v] = -1;
		return ecc;
	};
	for (int start0 = 0; start0 < n; start0++) {
		if (done[start0]) continue;
		// minimum-degree node of this component
		int s = start0;
		{
			std::vector<int> comp{start0};
			std::vector<char> in(0);
			std::vector<int> st{start0};
			level[start0] = 0;
			size_t h = 0;
			while (h < comp.size()) {
				const int v = comp[h++];
				for (int k = ptr[v]; k < ptr[v + 1]; k++)
					if (level[adj[k]] < 0 && !done[adj[k]]) { level[adj[k]] = 0; comp.push_back(adj[k]); }
			}
			for (int v : comp) {
				level[v] = -1;
				if (deg[v] < deg[s] || (deg[v] == deg[s] && v < s)) s = v;
			}
		}
		// George-Liu pseudo-peripheral node
		std::vector<int> last;
		int ecc = bfs_levels(s, last);
		for (int it = 0; it < 8; it++) {
			int best = last[0];
			for (int v : last)
				if (deg[v] < deg[best]) best = v;
			std::vector<int> last2;
			const int e2 = bfs_levels(best, last2);
			if (e2 > ecc) { ecc = e2; s = best; last = last2; }
			else break;
		}
		// Cuthill-McKee from s
		const size_t base = order.size();
		order.push_back(s);
		done[s] = 1;
		for (size_t h = base; h < order.size(); h++) {
			const int v = order[h];
			std::vector<int> nb;
			for (int k = ptr[v]; k < ptr[v + 1]; k++)
				if (!done[adj[k]]) { nb.push_back(adj[k]); done[adj[k]] = 1; }
			std::sort(nb.begin(), nb.end(), [&](int a, int b) { return deg[a] < deg[b] || (deg[a] == deg[b] && a < b); });
			for (int w : nb) order.push_back(w);
		}
	}
	std::reverse(order.begin(), order.end());
	return order;
}

int HostMesh::build(std::string *err)
{
	// ---- edge matching ----
	std::vector<EdgeRef> e = sorted_edges(nelem, nnode, inpoel);
	esuel.assign(4 * (size_t)nelem, std::numeric_limits<int>::min());
	for (int i = 0; i < nelem; i++)
		for (int j = 0; j < nnode[i]; j++) esuel[4 * i + j] = kUnmatched;
	std::vector<int> bnd_edge_idx;  // indices into e of edges with a single owner
	for (size_t k = 0; k < e.size();) {
		size_t k2 = k + 1;
		while (k2 < e.size() && e[k2].key == e[k].key) k2++;
		if (k2 - k == 2) {
			esuel[4 * e[k].cell + e[k].local] = e[k + 1].cell;
			esuel[4 * e[k + 1].cell + e[k + 1].local] = e[k].cell;
		} else if (k2 - k == 1) {
			bnd_edge_idx.push_back((int)k);
		} else {
			if (err) *err = "non-manifold edge shared by more than two cells";
			return 1;
		}
		k = k2;
	}
	// ---- boundary faces, in input order, oriented with their host cell ----
	std::unordered_map<uint64_t, int> bmap;
	bmap.reserve(bnd_edge_idx.size() * 2);
	for (int k : bnd_edge_idx) bmap[e[k].key] = k;
	if ((int)bnd_edge_idx.size() != nbface) {
		if (err) *err = "number of boundary faces does not match the unmatched cell edges";
		return 2;
	}
	ninface = 0;
	for (int i = 0; i < nelem; i++)
		for (int j = 0; j < nnode[i]; j++)
			if (esuel[4 * i + j] > i) ninface++;
	naface = nbface + ninface;
	face_l.assign(naface, 0); face_r.assign(naface, 0);
	face_n0.assign(naface, 0); face_n1.assign(naface, 0);
	face_sl.assign(naface, 0); face_sr.assign(naface, -1);
	elemface.assign(4 * (size_t)nelem, -1);
	for (int f = 0; f < nbface; f++) {
		auto it = bmap.find(edge_key(bface[2 * f], bface[2 * f + 1]));
		if (it == bmap.end()) {
			if (err) *err = "boundary face " + std::to_string(f) + " is not an edge of exactly one cell";
			return 3;
		}
		const EdgeRef &r = e[it->second];
		bmap.erase(it);
		const int h = r.cell, j = r.local;
		bface[2 * f] = inpoel[4 * h + j];
		bface[2 * f + 1] = inpoel[4 * h + (j + 1) % nnode[h]];
		face_l[f] = h; face_r[f] = -1 - f;
		face_n0[f] = bface[2 * f]; face_n1[f] = bface[2 * f + 1];
		face_sl[f] = j;
		esuel[4 * h + j] = -1 - f;
		elemface[4 * h + j] = f;
	}
	int fi = nbface;
	for (int i = 0; i < nelem; i++)
		for (int j = 0; j < nnode[i]; j++) {
			const int nb = esuel[4 * i + j];
			if (nb > i) {
				face_l[fi] = i; face_r[fi] = nb;
				face_n0[fi] = inpoel[4 * i + j];
				face_n1[fi] = inpoel[4 * i + (j + 1) % nnode[i]];
				face_sl[fi] = j;
				int jr = -1;
				for (int q = 0; q < nnode[nb]; q++)
					if (esuel[4 * nb + q] == i && inpoel[4 * nb + q] == face_n1[fi]) jr = q;
				if (jr < 0) {
					if (err) *err = "inconsistent cell orientation across an interior face";
					return 4;
				}
				face_sr[fi] = jr;
				elemface[4 * i + j] = fi;
				elemface[4 * nb + jr] = fi;
				fi++;
			}
		}
	// ---- geometry ----
	area.assign(nelem, 0.0);
	cc.assign(2 * (size_t)nelem, 0.0);
	for (int i = 0; i < nelem; i++) {
		area[i] = cell_area(coords.data(), &inpoel[4 * i], nnode[i]);
		for (int d = 0; d < 2; d++) {
			double s = 0;
			for (int j = 0; j < nnode[i]; j++) s += coords[2 * inpoel[4 * i + j] + d];
			cc[2 * i + d] = s / (double)nnode[i];
		}
	}
	fnorm.assign(3 * (size_t)naface, 0.0);
	fc.assign(2 * (size_t)naface, 0.0);
	for (int f = 0; f < naface; f++) {
		const double x0 = coords[2 * face_n0[f]], y0 = coords[2 * face_n0[f] + 1];
		const double x1 = coords[2 * face_n1[f]], y1 = coords[2 * face_n1[f] + 1];
		const double nx = y1 - y0, ny = -(x1 - x0);
		const double len = std::sqrt(nx * nx + ny * ny);
		fnorm[3 * f] = nx / len; fnorm[3 * f + 1] = ny / len; fnorm[3 * f + 2] = len;
		fc[2 * f] = (x0 + x1) / 2; fc[2 * f + 1] = (y0 + y1) / 2;
	}
	gc.assign(2 * (size_t)nbface, 0.0);
	for (int f = 0; f < nbface; f++)
		for (int d = 0; d < 2; d++) gc[2 * f + d] = 2.0 * fc[2 * f + d] - cc[2 * face_l[f] + d];
	// ---- greedy colouring of the interior-face adjacency, in cell order ----
	color.assign(nelem, -1);
	ncolors = 0;
	for (int i = 0; i < nelem; i++) {
		unsigned used = 0;
		for (int j = 0; j < nnode[i]; j++) {
			const int nb = esuel[4 * i + j];
			if (nb >= 0 && color[nb] >= 0) used |= 1u << color[nb];
		}
		int c = 0;
		while (used & (1u << c)) c++;
		color[i] = c;
		ncolors = std::max(ncolors, c + 1);
	}
	color_ptr.assign(ncolors + 1, 0);
	for (int i = 0; i < nelem; i++) color_ptr[color[i] + 1]++;
	for (int c = 0; c < ncolors; c++) color_ptr[c + 1] += color_ptr[c];
	color_cells.assign(nelem, 0);
	{
		std::vector<int> fill(color_ptr.begin(), color_ptr.end() - 1);
		for (int i = 0; i < nelem; i++) color_cells[fill[color[i]]++] = i;
	}
	return check(err);
}

int HostMesh::check(std::string *err) const
{
	for (int i = 0; i < nelem; i++) {
		if (!(area[i] > 0)) {
			if (err) *err = "cell " + std::to_string(i) + " has non-positive area";
			return 5;
		}
		for (int j = 0; j < nnode[i]; j++)
			if (esuel[4 * i + j] == kUnmatched) {
				if (err) *err = "cell " + std::to_string(i) + " has an unmatched edge";
				return 6;
			}
	}
	return 0;
}

int mesh_from_arrays(HostMesh &m, int npoin, const double *coords, int nelem, const int *nnode, const int *inpoel,
                     int nbface, const int *bface, const int *btag, int reorder, std::string *err)
{
	if (npoin <= 0 || nelem <= 0 || nbface < 0 || !coords || !nnode || !inpoel || (nbface > 0 && (!bface || !btag))) {
		if (err) *err = "invalid mesh description";
		return 1;
	}
	m = HostMesh();
	m.npoin = npoin; m.nelem = nelem; m.nbface = nbface;
	m.coords.assign(coords, coords + 2 * (size_t)npoin);
	m.nnode.assign(nnode, nnode + nelem);
	m.inpoel.assign(4 * (size_t)nelem, -1);
	for (int i = 0; i < nelem; i++) {
		if (nnode[i] != 3 && nnode[i] != 4) {
			if (err) *err = "only triangles and quadrilaterals are supported";
			return 1;
		}
		for (int j = 0; j < nnode[i]; j++) {
			const int p = inpoel[4 * i + j];
			if (p < 0 || p >= npoin) {
				if (err) *err = "node index out of range";
				return 1;
			}
			m.inpoel[4 * i + j] = p;
		}
		if (cell_area(m.coords.data(), &m.inpoel[4 * i], nnode[i]) < 0) std::reverse(&m.inpoel[4 * i], &m.inpoel[4 * i] + nnode[i]);
	}
	m.bface.assign(bface, bface + 2 * (size_t)nbface);
	m.btag.assign(btag, btag + nbface);
	m.perm.resize(nelem);
	std::iota(m.perm.begin(), m.perm.end(), 0);
	if (reorder == 1) {
		std::vector<EdgeRef> e = sorted_edges(nelem, m.nnode, m.inpoel);
		std::vector<int> deg(nelem, 0);
		std::vector<std::pair<int, int>> pairs;
		for (size_t k = 0; k + 1 < e.size(); k++)
			if (e[k].key == e[k + 1].key) pairs.push_back({e[k].cell, e[k + 1].cell});
		std::vector<int> ptr(nelem + 1, 0), adj(2 * pairs.size());
		for (auto &p : pairs) { ptr[p.first + 1]++; ptr[p.second + 1]++; }
		for (int i = 0; i < nelem; i++) ptr[i + 1] += ptr[i];
		std::vector<int> fill(ptr.begin(), ptr.end() - 1);
		for (auto &p : pairs) { adj[fill[p.first]++] = p.second; adj[fill[p.second]++] = p.first; }
		for (int i = 0; i < nelem; i++) std::sort(adj.begin() + ptr[i], adj.begin() + ptr[i + 1]);
		m.perm = rcm_order(nelem, ptr, adj);
		std::vector<int> nn(nelem), ip(4 * (size_t)nelem);
		for (int k = 0; k < nelem; k++) {
			nn[k] = m.nnode[m.perm[k]];
			for (int j = 0; j < 4; j++) ip[4 * k + j] = m.inpoel[4 * m.perm[k] + j];
		}
		m.nnode.swap(nn);
		m.inpoel.swap(ip);
	}
	return m.build(err);
}

RawMesh gen_channel_bump(int nx, int ny, double split_frac, uint64_t seed)
{
	RawMesh r;
	r.npoin = (nx + 1) * (ny + 1);
	r.coords.resize(2 * (size_t)r.npoin);
	for (int j = 0; j <= ny; j++)
		for (int i = 0; i <= nx; i++) {
			const double x = -1.5 + 3.0 * i / nx;
			const double yb = 0.0625 * std::exp(-25.0 * x * x);
			const double y = yb + (0.8 - yb) * (double)j / ny;
			r.coords[2 * (j * (nx + 1) + i)] = x;
			r.coords[2 * (j * (nx + 1) + i) + 1] = y;
		}
	const int nq = nx * ny;
	const int nsplit = (int)std::lround(split_frac * nq);
	uint64_t s = seed;
	std::vector<int> idx(nq);
	std::iota(idx.begin(), idx.end(), 0);
	for (int k = nq - 1; k > 0; k--) {
		const int t = (int)(splitmix64(s) % (uint64_t)(k + 1));
		std::swap(idx[k], idx[t]);
	}
	std::vector<int> split(nq, 0);
	for (int k = 0; k < nsplit; k++) split[idx[k]] = 1 + (int)(splitmix64(s) & 1u);
	auto node = [&](int i, int j) { return j * (nx + 1) + i; };
	for (int j = 0; j < ny; j++)
		for (int i = 0; i < nx; i++) {
			const int q = j * nx + i;
			const int a = node(i, j), b = node(i + 1, j), c = node(i + 1, j + 1), d = node(i, j + 1);
			if (!split[q]) {
				r.nnode.push_back(4);
				r.inpoel.insert(r.inpoel.end(), {a, b, c, d});
			} else if (split[q] == 1) {
				r.nnode.push_back(3); r.inpoel.insert(r.inpoel.end(), {a, b, c, -1});
				r.nnode.push_back(3); r.inpoel.insert(r.inpoel.end(), {a, c, d, -1});
			} else {
				r.nnode.push_back(3); r.inpoel.insert(r.inpoel.end(), {a, b, d, -1});
				r.nnode.push_back(3); r.inpoel.insert(r.inpoel.end(), {b, c, d, -1});
			}
		}
	r.nelem = (int)r.nnode.size();
	for (int i = 0; i < nx; i++) { r.bface.insert(r.bface.end(), {node(i, 0), node(i + 1, 0)}); r.btag.push_back(1); }
	for (int j = 0; j < ny; j++) { r.bface.insert(r.bface.end(), {node(nx, j), node(nx, j + 1)}); r.btag.push_back(2); }
	for (int i = 0; i < nx; i++) { r.bface.insert(r.bface.end(), {node(i + 1, ny), node(i, ny)}); r.btag.push_back(3); }
	for (int j = 0; j < ny; j++) { r.bface.insert(r.bface.end(), {node(0, j + 1), node(0, j)}); r.btag.push_back(4); }
	r.nbface = (int)r.btag.size();
	return r;
}

namespace {
double naca0012_half(double x)
{
	if (x < 0) x = 0;
	return 0.6 * (0.2969 * std::sqrt(x) - 0.1260 * x - 0.3516 * x * x + 0.2843 * x * x * x - 0.1036 * x * x * x * x);
}
}  // namespace

RawMesh gen_naca_ogrid(int nc, int nr, double rfar, int nbl, double h0, double gbl, int tri_from, uint64_t seed)
{
	const double PI = 3.14159265358979323846;
	RawMesh r;
	// airfoil points, counter-clockwise from the trailing edge
	std::vector<double> px(nc), py(nc), th(nc);
	for (int i = 0; i < nc; i++) {
		th[i] = 2.0 * PI * i / nc;
		const double x = 0.5 * (1.0 + std::cos(th[i]));
		const double yt = naca0012_half(x);
		px[i] = x;
		py[i] = (i == 0 || 2 * i == nc) ? 0.0 : (2 * i < nc ? yt : -yt);
	}
	// outward unit normals by central differences, lightly smoothed
	std::vector<double> nx(nc), ny(nc);
	for (int i = 0; i < nc; i++) {
		const int ip = (i + 1) % nc, im = (i + nc - 1) % nc;
		const double tx = px[ip] - px[im], ty = py[ip] - py[im];
		const double l = std::sqrt(tx * tx + ty * ty);
		nx[i] = ty / l; ny[i] = -tx / l;
	}
	for (int it = 0; it < 4; it++) {
		std::vector<double> ax(nc), ay(nc);
		for (int i = 0; i < nc; i++) {
			const int ip = (i + 1) % nc, im = (i + nc - 1) % nc;
			ax[i] = 0.5 * nx[i] + 0.25 * (nx[ip] + nx[im]);
			ay[i] = 0.5 * ny[i] + 0.25 * (ny[ip] + ny[im]);
			const double l = std::sqrt(ax[i] * ax[i] + ay[i] * ay[i]);
			ax[i] /= l; ay[i] /= l;
		}
		nx.swap(ax); ny.swap(ay);
	}
	// far-field angles: half normal direction, half the uniform O-grid angle (monotone)
	std::vector<double> phi(nc);
	double prev = 0;
	for (int i = 0; i < nc; i++) {
		double a = std::atan2(ny[i], nx[i]);
		while (a < prev - PI) a += 2 * PI;
		while (a > prev + PI) a -= 2 * PI;
		if (i == 0) a = 0;
		prev = a;
		phi[i] = 0.5 * a + 0.5 * th[i];
	}
	// ring distances
	const double D = rfar - 0.5;
	std::vector<double> d(nr + 1, 0.0);
	if (nbl <= 0) {
		const double hh = D * (gbl - 1.0) / (std::pow(gbl, nr) - 1.0);
		for (int k = 1; k <= nr; k++) d[k] = d[k - 1] + hh * std::pow(gbl, k - 1);
	} else {
		for (int k = 1; k <= nbl; k++) d[k] = d[k - 1] + h0 * std::pow(gbl, k - 1);
		const double hl = h0 * std::pow(gbl, nbl - 1);
		const int no = nr - nbl;
		double lo = 1.0 + 1e-12, hi = 2.0;
		for (int it = 0; it < 200; it++) {
			const double g = 0.5 * (lo + hi);
			const double tot = hl * g * (std::pow(g, no) - 1.0) / (g - 1.0);
			if (d[nbl] + tot > D) hi = g; else lo = g;
		}
		const double g2 = 0.5 * (lo + hi);
		for (int k = nbl + 1; k <= nr; k++) d[k] = d[k - 1] + hl * std::pow(g2, k - nbl);
		const double sc = (D - d[nbl]) / (d[nr] - d[nbl]);
		for (int k = nbl + 1; k <= nr; k++) d[k] = d[nbl] + (d[k] - d[nbl]) * sc;
	}
	const double dblend = 2.0;
	r.npoin = nc * (nr + 1);
	r.coords.resize(2 * (size_t)r.npoin);
	for (int k = 0; k <= nr; k++) {
		const double s = d[k] / D;
		const double t = std::min(1.0, d[k] / dblend);
		const double w = k == nr ? 1.0 : t * t * (3.0 - 2.0 * t);
		for (int i = 0; i < nc; i++) {
			const double qx = 0.5 + rfar * std::cos(phi[i]), qy = rfar * std::sin(phi[i]);
			const double ax = px[i] + d[k] * nx[i], ay = py[i] + d[k] * ny[i];
			const double bx = px[i] + s * (qx - px[i]), by = py[i] + s * (qy - py[i]);
			r.coords[2 * ((size_t)k * nc + i)] = (1 - w) * ax + w * bx;
			r.coords[2 * ((size_t)k * nc + i) + 1] = (1 - w) * ay + w * by;
		}
	}
	auto node = [&](int i, int k) { return k * nc + (i % nc); };
	uint64_t sd = seed;
	for (int k = 0; k < nr; k++)
		for (int i = 0; i < nc; i++) {
			// (i,k) -> (i,k+1) -> (i+1,k+1) -> (i+1,k) is counter-clockwise for a CCW airfoil
			const int a = node(i, k), b = node(i, k + 1), c = node(i + 1, k + 1), e = node(i + 1, k);
			if (k < tri_from) {
				r.nnode.push_back(4);
				r.inpoel.insert(r.inpoel.end(), {a, b, c, e});
			} else if (splitmix64(sd) & 1u) {
				r.nnode.push_back(3); r.inpoel.insert(r.inpoel.end(), {a, b, c, -1});
				r.nnode.push_back(3); r.inpoel.insert(r.inpoel.end(), {a, c, e, -1});
			} else {
				r.nnode.push_back(3); r.inpoel.insert(r.inpoel.end(), {a, b, e, -1});
				r.nnode.push_back(3); r.inpoel.insert(r.inpoel.end(), {b, c, e, -1});
			}
		}
	r.nelem = (int)r.nnode.size();
	for (int i = 0; i < nc; i++) { r.bface.insert(r.bface.end(), {node(i, 0), node(i + 1, 0)}); r.btag.push_back(2); }
	for (int i = 0; i < nc; i++) { r.bface.insert(r.bface.end(), {node(i, nr), node(i + 1, nr)}); r.btag.push_back(4); }
	r.nbface = (int)r.btag.size();
	return r;
}

/* Hybrid NACA 0012 mesh with near-isotropic outer triangles.  Surface: nc
 * points, x = (1 - beta) cosine spacing + beta uniform spacing (beta bounds
 * the clustering at the leading and trailing edges).  Boundary layer: nbl quad
 * rings extruded with heights h0 g^k along the surface normals, lightly
 * smoothed (the cells stay close to orthogonal up to the trailing-edge fan).
 * Outer region: each ring is the previous one offset along its
 * normals by sqrt(3)/2 times its mean edge length (near-equilateral
 * triangles, geometric growth), then resampled by arc length at parameters
 * that drift by 3 % per ring from the boundary layer's distribution towards
 * uniform spacing; rings are added until every node is at least rfar from
 * mid-chord.  Quads between outer rings are split along the shorter diagonal. */
RawMesh gen_naca_hybrid(int nc, int nbl, double h0, double gbl, double rfar, double beta)
{
	const double PI = 3.14159265358979323846;
	RawMesh r;
	std::vector<double> px(nc), py(nc);
	for (int i = 0; i < nc; i++) {
		const double t = (double)i / nc;
		const double xc = 0.5 * (1.0 + std::cos(2.0 * PI * t));
		const double xu = t <= 0.5 ? 1.0 - 2.0 * t : 2.0 * t - 1.0;
		const double x = (1.0 - beta) * xc + beta * xu;
		const double yt = naca0012_half(x);
		px[i] = x;
		py[i] = (i == 0 || 2 * i == nc) ? 0.0 : (2 * i < nc ? yt : -yt);
	}
	// outward unit normals of a closed counter-clockwise ring, then `passes`
	// rounds of [1/4 1/2 1/4] smoothing along the ring
	auto normals = [&](const std::vector<double> &x, const std::vector<double> &y, std::vector<double> &nx,
	                   std::vector<double> &ny, int passes) {
		nx.assign(nc, 0.0);
		ny.assign(nc, 0.0);
		for (int i = 0; i < nc; i++) {
			const int ip = (i + 1) % nc, im = (i + nc - 1) % nc;
			const double tx = x[ip] - x[im], ty = y[ip] - y[im];
			const double l = std::sqrt(tx * tx + ty * ty);
			nx[i] = ty / l;
			ny[i] = -tx / l;
		}
		std::vector<double> ax(nc), ay(nc);
		for (int it = 0; it < passes; it++) {
			for (int i = 0; i < nc; i++) {
				const int ip = (i + 1) % nc, im = (i + nc - 1) % nc;
				ax[i] = 0.5 * nx[i] + 0.25 * (nx[ip] + nx[im]);
				ay[i] = 0.5 * ny[i] + 0.25 * (ny[ip] + ny[im]);
				const double l = std::sqrt(ax[i] * ax[i] + ay[i] * ay[i]);
				ax[i] /= l;
				ay[i] /= l;
			}
			nx.swap(ax);
			ny.swap(ay);
		}
	};
	std::vector<std::vector<double>> rx, ry;  // rings, 0 = the surface
	rx.push_back(px);
	ry.push_back(py);
	std::vector<double> nx, ny;
	normals(px, py, nx, ny, 4);
	double d = 0.0;
	for (int k = 1; k <= nbl; k++) {
		d += h0 * std::pow(gbl, k - 1);
		std::vector<double> x(nc), y(nc);
		for (int i = 0; i < nc; i++) { x[i] = px[i] + d * nx[i]; y[i] = py[i] + d * ny[i]; }
		rx.push_back(x);
		ry.push_back(y);
	}
	// arc-length parameter (fraction of the perimeter from node 0) of a closed ring's nodes
	auto arclen = [&](const std::vector<double> &x, const std::vector<double> &y, std::vector<double> &cs) {
		cs.assign(nc + 1, 0.0);
		for (int i = 0; i < nc; i++) cs[i + 1] = cs[i] + std::hypot(x[(i + 1) % nc] - x[i], y[(i + 1) % nc] - y[i]);
		return cs[nc];
	};
	std::vector<double> cs, s(nc);
	{
		const double P = arclen(rx.back(), ry.back(), cs);
		for (int i = 0; i < nc; i++) s[i] = cs[i] / P;
	}
	const int max_rings = 100000;
	for (int it = 0; it < max_rings; it++) {
		const std::vector<double> &x = rx.back(), &y = ry.back();
		double rmin = 1e300;
		for (int i = 0; i < nc; i++) rmin = std::min(rmin, std::hypot(x[i] - 0.5, y[i]));
		if (rmin >= rfar) break;
		const double h = arclen(x, y, cs) / nc;
		normals(x, y, nx, ny, 2);
		std::vector<double> ox(nc), oy(nc), X(nc), Y(nc);
		for (int i = 0; i < nc; i++) {
			ox[i] = x[i] + 0.8660254037844386 * h * nx[i];
			oy[i] = y[i] + 0.8660254037844386 * h * ny[i];
		}
		const double P = arclen(ox, oy, cs);
		int seg = 0;
		for (int i = 0; i < nc; i++) {
			s[i] = 0.97 * s[i] + 0.03 * ((double)i / nc);
			const double t = s[i] * P;
			while (seg < nc - 1 && cs[seg + 1] < t) seg++;
			const double f = cs[seg + 1] > cs[seg] ? (t - cs[seg]) / (cs[seg + 1] - cs[seg]) : 0.0;
			const int j = (seg + 1) % nc;
			X[i] = ox[seg] + f * (ox[j] - ox[seg]);
			Y[i] = oy[seg] + f * (oy[j] - oy[seg]);
		}
		rx.push_back(X);
		ry.push_back(Y);
	}
	const int nr = (int)rx.size() - 1;
	r.npoin = nc * (nr + 1);
	r.coords.resize(2 * (size_t)r.npoin);
	for (int k = 0; k <= nr; k++)
		for (int i = 0; i < nc; i++) {
			r.coords[2 * ((size_t)k * nc + i)] = rx[k][i];
			r.coords[2 * ((size_t)k * nc + i) + 1] = ry[k][i];
		}
	auto node = [&](int i, int k) { return k * nc + (i % nc); };
	auto dist2 = [&](int a, int b) {
		const double dx = r.coords[2 * (size_t)a] - r.coords[2 * (size_t)b];
		const double dy = r.coords[2 * (size_t)a + 1] - r.coords[2 * (size_t)b + 1];
		return dx * dx + dy * dy;
	};
	for (int k = 0; k < nr; k++)
		for (int i = 0; i < nc; i++) {
			// (i,k) -> (i,k+1) -> (i+1,k+1) -> (i+1,k) is counter-clockwise
			const int a = node(i, k), b = node(i, k + 1), c = node(i + 1, k + 1), e = node(i + 1, k);
			if (k < nbl) {
				r.nnode.push_back(4);
				r.inpoel.insert(r.inpoel.end(), {a, b, c, e});
			} else if (dist2(a, c) <= dist2(b, e)) {
				r.nnode.push_back(3); r.inpoel.insert(r.inpoel.end(), {a, b, c, -1});
				r.nnode.push_back(3); r.inpoel.insert(r.inpoel.end(), {a, c, e, -1});
			} else {
				r.nnode.push_back(3); r.inpoel.insert(r.inpoel.end(), {a, b, e, -1});
				r.nnode.push_back(3); r.inpoel.insert(r.inpoel.end(), {b, c, e, -1});
			}
		}
	r.nelem = (int)r.nnode.size();
	for (int i = 0; i < nc; i++) { r.bface.insert(r.bface.end(), {node(i, 0), node(i + 1, 0)}); r.btag.push_back(2); }
	for (int i = 0; i < nc; i++) { r.bface.insert(r.bface.end(), {node(i, nr), node(i + 1, nr)}); r.btag.push_back(4); }
	r.nbface = (int)r.btag.size();
	return r;
}

namespace {
/* next "KEY=value" header of an SU2 file: the value as an integer (tags and
 * counts are numeric in the meshes this reader supports) */
bool su2_header(std::istream &in, const char *key, long &value, std::string *err)
{
	std::string tok;
	while (in >> tok) {
		const size_t eq = tok.find('=');
		if (eq == std::string::npos) continue;
		if (tok.compare(0, eq, key) != 0) continue;
		std::string v = tok.substr(eq + 1);
		if (v.empty() && !(in >> v)) break;
		try {
			value = std::stol(v);
		} catch (...) {
			if (err) *err = std::string("SU2: non-numeric value of ") + key + ": " + v;
			return false;
		}
		return true;
	}
	if (err) *err = std::string("SU2: missing ") + key;
	return false;
}
}  // namespace

int read_su2(const std::string &path, RawMesh &out, std::string *err)
{
	std::ifstream in(path);
	if (!in) {
		if (err) *err = "cannot open " + path;
		return 1;
	}
	out = RawMesh();
	long ndim = 0, nelem = 0, npoin = 0, nmark = 0;
	if (!su2_header(in, "NDIME", ndim, err)) return 2;
	if (ndim != 2) {
		if (err) *err = "SU2: mesh is not 2-dimensional";
		return 2;
	}
	if (!su2_header(in, "NELEM", nelem, err)) return 2;
	out.nelem = (int)nelem;
	out.nnode.resize(nelem);
	out.inpoel.assign(4 * (size_t)nelem, -1);
	for (long k = 0; k < nelem; k++) {
		int type;
		if (!(in >> type)) { if (err) *err = "SU2: truncated element list"; return 3; }
		const int nn = type == 5 ? 3 : type == 9 ? 4 : 0;
		if (!nn) {
			if (err) *err = "SU2: unknown element type " + std::to_string(type);
			return 3;
		}
		out.nnode[k] = nn;
		for (int q = 0; q < nn; q++) in >> out.inpoel[4 * k + q];
		long idx;
		in >> idx;
	}
	if (!su2_header(in, "NPOIN", npoin, err)) return 2;
	out.npoin = (int)npoin;
	out.coords.resize(2 * (size_t)npoin);
	{
		// each point line: x y [index]; the index is optional
		std::string line;
		std::getline(in, line);
		for (long k = 0; k < npoin; k++) {
			if (!std::getline(in, line)) { if (err) *err = "SU2: truncated point list"; return 3; }
			std::istringstream ls(line);
			if (!(ls >> out.coords[2 * k] >> out.coords[2 * k + 1])) {
				if (err) *err = "SU2: bad point line " + std::to_string(k);
				return 3;
			}
		}
	}
	if (!su2_header(in, "NMARK", nmark, err)) return 2;
	for (long mk = 0; mk < nmark; mk++) {
		long tag = 0, ne = 0;
		if (!su2_header(in, "MARKER_TAG", tag, err)) return 2;
		if (!su2_header(in, "MARKER_ELEMS", ne, err)) return 2;
		for (long k = 0; k < ne; k++) {
			int type, a, b;
			if (!(in >> type >> a >> b) || type != 3) {
				if (err) *err = "SU2: boundary elements must be lines (type 3)";
				return 3;
			}
			out.bface.push_back(a);
			out.bface.push_back(b);
			out.btag.push_back((int)tag);
		}
	}
	out.nbface = (int)out.btag.size();
	for (int v : out.inpoel)
		if (v >= (int)npoin) {
			if (err) *err = "SU2: node index out of range";
			return 4;
		}
	return 0;
}

int read_gmsh2(const std::string &path, RawMesh &out, std::string *err)
{
	std::ifstream in(path);
	if (!in) {
		if (err) *err = "cannot open " + path;
		return 1;
	}
	out = RawMesh();
	std::unordered_map<long, int> nid;
	std::string line;
	while (std::getline(in, line)) {
		if (line.rfind("$Nodes", 0) == 0) {
			long n;
			in >> n;
			out.npoin = (int)n;
			out.coords.resize(2 * (size_t)n);
			for (long k = 0; k < n; k++) {
				long id;
				double x, y, z;
				in >> id >> x >> y >> z;
				nid[id] = (int)k;
				out.coords[2 * k] = x;
				out.coords[2 * k + 1] = y;
			}
		} else if (line.rfind("$Elements", 0) == 0) {
			long n;
			in >> n;
			for (long k = 0; k < n; k++) {
				long id;
				int type, ntags;
				in >> id >> type >> ntags;
				std::vector<long> tags(ntags);
				for (int t = 0; t < ntags; t++) in >> tags[t];
				int nn = type == 1 ? 2 : type == 2 ? 3 : type == 3 ? 4 : type == 15 ? 1 : -1;
				if (nn < 0) {
					if (err) *err = "unsupported Gmsh element type " + std::to_string(type);
					return 2;
				}
				std::vector<int> nodes(nn);
				for (int q = 0; q < nn; q++) {
					long v;
					in >> v;
					auto it = nid.find(v);
					if (it == nid.end()) {
						if (err) *err = "element refers to an unknown node";
						return 3;
					}
					nodes[q] = it->second;
				}
				if (type == 1) {
					out.bface.push_back(nodes[0]);
					out.bface.push_back(nodes[1]);
					out.btag.push_back(ntags > 0 ? (int)tags[0] : 0);
				} else if (type == 2 || type == 3) {
					out.nnode.push_back(nn);
					for (int q = 0; q < 4; q++) out.inpoel.push_back(q < nn ? nodes[q] : -1);
				}
			}
		}
	}
	out.nelem = (int)out.nnode.size();
	out.nbface = (int)out.btag.size();
	if (out.npoin == 0 || out.nelem == 0) {
		if (err) *err = "no nodes or cells found in " + path;
		return 4;
	}
	return 0;
}

}  // namespace fvg

namespace fvg {

int find_lines(HostMesh &h, double threshold)
{
	const int n = h.nelem;
	// neighbours of each cell ordered by decreasing weight (computeWeights)
	std::vector<std::array<std::pair<double, int>, 4>> w(n);
	std::vector<int> nreal(n, 0);
	for (int i = 0; i < n; i++) {
		double minw = 1e20;
		int k = 0;
		for (int j = 0; j < h.nnode[i]; j++) {
			const int nb = h.esuel[4 * i + j];
			if (nb < 0) continue;
			const double dx = h.cc[2 * i] - h.cc[2 * nb], dy = h.cc[2 * i + 1] - h.cc[2 * nb + 1];
			const double wt = 1.0 / std::sqrt(dx * dx + dy * dy);
			if (wt < minw) minw = wt;
			w[i][k++] = {wt, nb};
		}
		for (int a = 0; a < k; a++) w[i][a].first /= minw;
		std::stable_sort(w[i].begin(), w[i].begin() + k,
		                 [](const std::pair<double, int> &a, const std::pair<double, int> &b) { return a.first > b.first; });
		nreal[i] = k;
	}
	h.lines.clear();
	h.cell_line.assign(n, -1);
	for (int f = 0; f < h.nbface; f++) {
		const int b = h.face_l[f];
		if (h.cell_line[b] >= 0) continue;
		std::vector<int> line;
		int cur = b;
		while (true) {
			if (nreal[cur] == 0 || !(w[cur][0].first > threshold)) break;
			line.push_back(cur);
			h.cell_line[cur] = (int)h.lines.size();
			int next = -1;
			for (int j = 0; j < nreal[cur]; j++) {
				const int nb = w[cur][j].second;
				if (h.cell_line[nb] == -1 && w[cur][j].first > threshold) { next = nb; break; }
			}
			if (next < 0) break;
			cur = next;
		}
		if (line.size() > 1) h.lines.push_back(line);
		else if (line.size() == 1) h.cell_line[line[0]] = -1;
	}
	return (int)h.lines.size();
}

std::vector<int> periodic_map(const HostMesh &h, int bcm, int axis)
{
	std::vector<int> map(h.nbface, -1);
	if (bcm < 0 || axis < 0 || axis > 1) return map;
	const int ax = 1 - axis;
	auto centre = [&](int f) { return (h.coords[2 * h.bface[2 * f] + ax] + h.coords[2 * h.bface[2 * f + 1] + ax]) / 2.0; };
	for (int i = 0; i < h.nbface; i++) {
		if (h.btag[i] != bcm || map[i] > -1) continue;
		const double ci = centre(i);
		for (int j = i + 1; j < h.nbface; j++) {
			if (h.btag[j] != bcm || map[j] > -1) continue;
			if (std::fabs(ci - centre(j)) <= 1e-8) {
				map[i] = j;
				map[j] = i;
				break;
			}
		}
	}
	return map;
}

namespace {

/* Colours of a graph (adjacency lists, sorted, no self loops): DSatur (Brelaz
 * 1979: the uncoloured vertex with the most distinct neighbour colours goes
 * next, ties by degree then index, each vertex the smallest free colour), then
 * Kempe-chain interchanges that move every vertex of the last colour into a
 * lower one where a two-colour chain swap frees it; repeated while the last
 * colour empties.  On the part graph of the transonic NACA 0012 O-grid this
 * gives 4 colours where greedy colouring in part order gives 5.  Deterministic. */
std::vector<int> colour_parts(const std::vector<std::vector<int>> &adj)
{
	const int np = (int)adj.size();
	std::vector<int> col(np, -1);
	std::vector<std::vector<char>> seen(np);  // per vertex: neighbour colours present
	std::vector<int> sat(np, 0);
	std::set<std::tuple<int, int, int>> pq;  // (-saturation, -degree, index)
	for (int v = 0; v < np; v++) pq.insert({0, -(int)adj[v].size(), v});
	while (!pq.empty()) {
		const int v = std::get<2>(*pq.begin());
		pq.erase(pq.begin());
		int c = 0;
		while (c < (int)seen[v].size() && seen[v][c]) c++;
		col[v] = c;
		for (int u : adj[v]) {
			if (col[u] >= 0) continue;
			if ((int)seen[u].size() <= c) seen[u].resize(c + 1, 0);
			if (!seen[u][c]) {
				pq.erase({-sat[u], -(int)adj[u].size(), u});
				seen[u][c] = 1;
				sat[u]++;
				pq.insert({-sat[u], -(int)adj[u].size(), u});
			}
		}
	}
	int nc = 0;
	for (int c : col) nc = std::max(nc, c + 1);
	std::vector<int> mark(np, 0), stack;
	int stamp = 0;
	while (nc > 1) {
		const int top = nc - 1;
		bool all = true;
		for (int v = 0; v < np; v++) {
			if (col[v] != top) continue;
			bool moved = false;
			for (int a = 0; a < top && !moved; a++)
				for (int b = 0; b < top && !moved; b++) {
					if (a == b) continue;
					// the a/b chains through v's a-coloured neighbours
					stamp++;
					stack.clear();
					for (int j : adj[v])
						if (col[j] == a) { mark[j] = stamp; stack.push_back(j); }
					std::vector<int> chain = stack;
					while (!stack.empty()) {
						const int x = stack.back();
						stack.pop_back();
						for (int y : adj[x])
							if (mark[y] != stamp && (col[y] == a || col[y] == b)) {
								mark[y] = stamp;
								stack.push_back(y);
								chain.push_back(y);
							}
					}
					bool blocked = false;  // a b-neighbour of v in the chains: the swap frees no colour
					for (int j : adj[v])
						if (col[j] == b && mark[j] == stamp) blocked = true;
					if (blocked) continue;
					for (int x : chain) col[x] = col[x] == a ? b : a;
					col[v] = a;
					moved = true;
				}
			if (!moved) all = false;
		}
		if (!all) break;
		nc--;
	}
	return col;
}

}  // namespace

BlockOrder block_colour_order(const HostMesh &h, int part_size, int colouring)
{
	BlockOrder o;
	const int n = h.nelem;
	const size_t target = (size_t)std::max(part_size, 1);
	// parts grown breadth-first over the cell graph, each from the lowest-numbered
	// cell not yet in a part: compact in the cell graph, so the dependency chains
	// inside a part are about as long as the part is wide (in cells)
	// units that go into a part whole: a single cell, or a piece (at most
	// `target` cells) of a line of strongly coupled cells
	std::vector<int> unit_of(n, -1);
	std::vector<std::vector<int>> units;
	for (const auto &ln : h.lines)
		for (size_t a = 0; a < ln.size(); a += target) {
			units.emplace_back(ln.begin() + a, ln.begin() + std::min(ln.size(), a + target));
			for (int c : units.back()) unit_of[c] = (int)units.size() - 1;
		}
	for (int c = 0; c < n; c++)
		if (unit_of[c] < 0) {
			unit_of[c] = (int)units.size();
			units.push_back({c});
		}
	std::vector<int> pid(n, -1);
	std::vector<std::vector<int>> cells;
	std::vector<int> queue;
	queue.reserve(target);
	auto add_unit = [&](int u, int k) {
		for (int c : units[u]) {
			pid[c] = k;
			queue.push_back(c);
		}
	};
	for (int seed = 0; seed < n; seed++) {
		if (pid[seed] >= 0) continue;
		const int k = (int)cells.size();
		queue.clear();
		add_unit(unit_of[seed], k);
		for (size_t head = 0; head < queue.size() && queue.size() < target; head++) {
			const int c = queue[head];
			for (int j = 0; j < h.nnode[c] && queue.size() < target; j++) {
				const int nb = h.esuel[4 * c + j];
				if (nb >= 0 && pid[nb] < 0 && queue.size() + units[unit_of[nb]].size() <= target) add_unit(unit_of[nb], k);
			}
		}
		cells.push_back(queue);
		std::sort(cells.back().begin(), cells.back().end());
	}
	const int np = (int)cells.size();
	// colour the part adjacency graph: each colour is one launch of every sweep
	std::vector<std::vector<int>> padj(np);
	for (int f = h.nbface; f < h.naface; f++) {
		const int a = pid[h.face_l[f]], b = pid[h.face_r[f]];
		if (a != b) { padj[a].push_back(b); padj[b].push_back(a); }
	}
	for (auto &v : padj) {
		std::sort(v.begin(), v.end());
		v.erase(std::unique(v.begin(), v.end()), v.end());
	}
	std::vector<int> pcol(np, -1);
	if (colouring == 1) {
		pcol = colour_parts(padj);
	} else {
		// greedy in part order
		for (int k = 0; k < np; k++) {
			std::vector<char> used(64, 0);
			for (int j : padj[k])
				if (pcol[j] >= 0 && pcol[j] < 64) used[pcol[j]] = 1;
			int c = 0;
			while (used[c]) c++;
			pcol[k] = c;
		}
	}
	int nc = 0;
	for (int c : pcol) nc = std::max(nc, c + 1);
	o.nparts = np;
	o.ncolors = nc;
	o.part_ptr.push_back(0);
	o.cpart_ptr.assign(nc + 1, 0);
	o.lev_ptr.push_back(0);
	std::vector<int> level(n, 0);
	for (int c = 0; c < nc; c++) {
		for (int k = 0; k < np; k++) {
			if (pcol[k] != c) continue;
			// levels of the lower-triangular dependencies inside the part (cells in index order)
			int maxl = 0;
			for (int i : cells[k]) {
				int l = 0;
				for (int j = 0; j < h.nnode[i]; j++) {
					const int nb = h.esuel[4 * i + j];
					if (nb >= 0 && nb < i && pid[nb] == k) l = std::max(l, level[nb] + 1);
				}
				level[i] = l;
				maxl = std::max(maxl, l);
			}
			std::vector<int> sorted = cells[k];
			std::stable_sort(sorted.begin(), sorted.end(), [&](int a, int b) { return level[a] < level[b]; });
			const int base = (int)o.pos_cell.size();
			for (size_t q = 0; q < sorted.size(); q++) {
				if (q == 0 || level[sorted[q]] != level[sorted[q - 1]]) o.lev_pos.push_back(base + (int)q);
				o.pos_cell.push_back(sorted[q]);
			}
			// widest level
			for (size_t q = 0, s = 0; q <= sorted.size(); q++)
				if (q == sorted.size() || (q > 0 && level[sorted[q]] != level[sorted[q - 1]])) {
					o.max_width = std::max(o.max_width, (int)(q - s));
					s = q;
				}
			o.lev_ptr.push_back((int)o.lev_pos.size());
			o.part_ptr.push_back((int)o.pos_cell.size());
		}
		o.cpart_ptr[c + 1] = (int)o.part_ptr.size() - 1;
	}
	return o;
}

}  // namespace fvg
