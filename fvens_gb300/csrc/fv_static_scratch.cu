/*
 * fv_compute_residual_static: the residual evaluation of fv_compute_residual
 * (same kernels, same results) with its scratch -- primitive and ghost
 * states, gradients, reconstruction gradients, face fluxes and face spectral radii --
 * carved out of one file-scope device array instead of the buffers the
 * discretisation handle allocated for itself.
 *
 * Who needs it: a caller that has to keep the device memory of its
 * evaluation path fixed and allocation-free -- for example a host code whose
 * device memory is handed out by its own pool or a memory cap, and which
 * evaluates residuals of many discretisations one after another without
 * holding a scratch set per handle.  Neither this call nor its set-up calls
 * cudaMalloc, cudaFree or any allocating library routine; the array is part
 * of the library's device image.
 *
 * Set-up: the first call on a device, with that device current, looks up the
 * array's device address with cudaGetSymbolAddress (once per device; the
 * result is kept).  Make that first call before any stream capture.  The
 * device current at the call must be the one the handle was created on
 * (FV_ERR_INVALID otherwise).  The handle itself is only read: its own
 * scratch buffers stay untouched.
 *
 * Limit: the scratch of one evaluation must fit in kStaticScratchBytes
 * (64 MiB): larger discretisations (cells x batch) are rejected with
 * FV_ERR_INVALID.  Nothing in the array has to start at zero: every scratch
 * entry is written before it is read within one evaluation.
 *
 * Every call shares the one array: calls whose GPU work overlaps (on
 * different streams, or from different handles running concurrently) race on
 * it and give wrong results.  Order such calls on one stream or synchronise
 * between them.
 */
#include <mutex>
#include <string>
#include <vector>

#include "fv_abi_internal.hpp"

namespace {

constexpr size_t kStaticScratchBytes = size_t(64) << 20;

__device__ __align__(256) unsigned char g_residual_scratch[kStaticScratchBytes];

std::mutex g_mu;
std::vector<void *> g_scratch_addr;  // per device ordinal, set on the first call there

size_t round256(size_t x) { return (x + 255) & ~size_t(255); }

/* Lays the scratch of one evaluation out from base (NULL: sizes only);
 * returns the bytes used.  Sizes as the handle's own buffers (fv_disc_create). */
size_t carve(const fvg::DiscDev &d, int batch, bool lgrad, unsigned char *base, fvg::ResidualWork *w)
{
	const size_t B = batch, ne = d.nelem, nf = d.naface, nb = d.nbface > 0 ? d.nbface : 1;
	size_t off = 0;
	auto take = [&](auto **p, size_t n) {
		using T = std::remove_pointer_t<std::remove_reference_t<decltype(*p)>>;
		if (base) *p = reinterpret_cast<T *>(base + off);
		off = round256(off + n * sizeof(T));
	};
	fvg::ResidualWork tmp;
	fvg::ResidualWork &x = w ? *w : tmp;
	take(&x.prim, B * ne);
	take(&x.ghost_prim, B * nb);
	take(&x.ghost_cons, B * nb);
	take(&x.grad, 2 * B * ne);
	take(&x.lgrad, lgrad ? 2 * B * ne : 1);
	take(&x.fflux, B * nf);
	take(&x.spec, B * nf);
	return off;
}

}  // namespace

using namespace fvg;

extern "C" fv_status fv_compute_residual_static(fv_disc *D, const double *u, double *r, int gettimesteps, double *dt)
{
	if (!D || !u || !r || (gettimesteps && !dt)) { set_error("null argument"); return FV_ERR_INVALID; }
	const bool lg = recon_gradients(D->d.recon);
	const size_t need = carve(D->d, D->batch, lg, nullptr, nullptr);
	if (need > kStaticScratchBytes) {
		set_error("static residual scratch: this discretisation needs " + std::to_string(need) +
		          " bytes (cells x batch too large); the static array holds " + std::to_string(kStaticScratchBytes));
		return FV_ERR_INVALID;
	}
	int dev = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if (e) return cuda_status(e, "static residual scratch: current device");
	if (dev != D->device) {
		set_error("static residual scratch: the handle was created on device " + std::to_string(D->device) +
		          " but device " + std::to_string(dev) + " is current");
		return FV_ERR_INVALID;
	}
	void *base = nullptr;
	{
		std::lock_guard<std::mutex> lk(g_mu);
		if ((int)g_scratch_addr.size() <= dev) g_scratch_addr.resize(dev + 1, nullptr);
		if (!g_scratch_addr[dev]) {
			e = cudaGetSymbolAddress(&base, g_residual_scratch);
			if (e) return cuda_status(e, "static residual scratch: cudaGetSymbolAddress");
			g_scratch_addr[dev] = base;
		}
		base = g_scratch_addr[dev];
	}
	ResidualWork w;
	carve(D->d, D->batch, lg, static_cast<unsigned char *>(base), &w);
	const int before = D->kernels_launched;
	e = residual_launch(D, u, r, gettimesteps, dt, D->stream, &w);
	count_launches(D->kernels_launched - before);
	return cuda_status(e, "residual (static scratch)");
}
