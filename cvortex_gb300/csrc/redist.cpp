// redist.cpp -- cvtx_P3D_redistribute_on_grid / cvtx_P2D_redistribute_on_grid
// (reference src/P3D.cpp:508-634, src/P2D.cpp:283-404, with the helpers of
// src/redistribution_helper_funcs.cpp and src/array_methods.cpp).
//
// Grid set-up and the final strength filtering run on the host (O(cells));
// spreading the particles onto the grid and summing per grid point run on the
// GPU when an accelerator is enabled and the redistribution function is one
// of this library's (redist.cu), else on the host. The algorithm and its
// order of operations are described in redist.h.
//
// The output order is the depth-first order of the reference's octree /
// quadtree without building a tree: that order is ascending Morton order of
// the grid keys, so one sort of the keys gives it.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <parallel/algorithm>
#include <string>
#include <vector>

#include "cvortex/libcvtx.h"
#include "redist.h"
#include "runtime.h"

namespace cvtx {

bool redist_grid(int dims, const float* pos, int n, const cvtx_RedistFunc* f, float gd,
	RedistGrid* g)
{
	g->dims = dims;
	g->gd = gd;
	g->rgd = 1.f / gd;
	g->radius = int(std::round(f->radius));
	g->bits = dims == 3 ? 21 : 31;
	float mn[3] = {0.f, 0.f, 0.f};
	double sum[3] = {0.0, 0.0, 0.0};
	for (int d = 0; d < dims; ++d) mn[d] = n > 0 ? pos[d] : 0.f;
	for (int i = 0; i < n; ++i)
		for (int d = 0; d < dims; ++d) {
			const float x = pos[size_t(i) * dims + d];
			mn[d] = mn[d] > x ? x : mn[d];
			sum[d] += double(x);
		}
	const float shift = float(g->radius) * gd;
	double hi[3] = {0.0, 0.0, 0.0};
	for (int d = 0; d < dims; ++d) {
		const float mean = float(sum[d] / double(n));
		const float lo = mn[d] - shift;
		const float dc = std::round((mean - lo) / gd) + 5.f;
		g->min[d] = mean - dc * gd;
		hi[d] = 0.0;
	}
	// the largest key must fit the Morton code
	for (int i = 0; i < n; ++i)
		for (int d = 0; d < dims; ++d) {
			const double k = double((pos[size_t(i) * dims + d] - g->min[d]) * g->rgd);
			hi[d] = std::max(hi[d], k);
		}
	const double lim = double(1u << g->bits) - double(g->radius) - 2.0;
	for (int d = 0; d < dims; ++d)
		if (!(hi[d] < lim)) return false;
	return true;
}

namespace {

struct Entry { uint64_t code; uint64_t order; };

// The contribution of particle i to stencil point s (code, strength); false if
// it is exactly zero. Each operation rounds separately (the translation unit
// is compiled without contraction), matching the GPU kernel.
inline bool contribution(const RedistGrid& g, const cvtx_RedistFunc* f, const float* pos,
	const float* str, int i, int s, uint64_t* code, float* val)
{
	const int w = 2 * g.radius + 1;
	int off[3];
	if (g.dims == 3) { off[0] = s / (w * w); off[1] = (s / w) % w; off[2] = s % w; }
	else { off[0] = s / w; off[1] = s % w; off[2] = 0; }
	float frac = 1.f;
	uint32_t key[3] = {0u, 0u, 0u};
	for (int d = 0; d < g.dims; ++d) {
		const float x = pos[size_t(i) * g.dims + d];
		const float t = (x - g.min[d]) * g.rgd;
		key[d] = uint32_t(int64_t(std::round(t))) + uint32_t(off[d] - g.radius);
		const float np = g.min[d] + g.gd * float(key[d]);
		const float u = std::fabs((x - np) * g.rgd);
		frac = d == 0 ? f->func(u) : frac * f->func(u);
	}
	bool nz = false;
	const int nc = g.dims == 3 ? 3 : 1;
	for (int c = 0; c < nc; ++c) {
		val[c] = str[size_t(i) * nc + c] * frac;
		nz = nz || val[c] != 0.f;
	}
	*code = g.dims == 3 ? (spread3(key[0]) | (spread3(key[1]) << 1) | (spread3(key[2]) << 2))
		: (spread2(key[0]) | (spread2(key[1]) << 1));
	return nz;
}

}  // namespace

void redist_cells_host(const RedistGrid& g, const cvtx_RedistFunc* f, const float* pos,
	const float* str, int n, RedistCells* out)
{
	const int w = 2 * g.radius + 1;
	const int S = g.dims == 3 ? w * w * w : w * w;
	const int nc = g.dims == 3 ? 3 : 1;
	const size_t m = size_t(n) * size_t(S);
	std::vector<Entry> e(m);
	std::vector<float> v(m * nc);
	std::vector<char> keep(m);
#pragma omp parallel for schedule(static)
	for (long long i = 0; i < n; ++i)
		for (int s = 0; s < S; ++s) {
			const size_t j = size_t(i) * S + s;
			keep[j] = contribution(g, f, pos, str, int(i), s, &e[j].code, &v[j * nc]) ? 1 : 0;
			e[j].order = j;
		}
	size_t k = 0;
	for (size_t j = 0; j < m; ++j)
		if (keep[j]) e[k++] = e[j];
	e.resize(k);
	__gnu_parallel::sort(e.begin(), e.end(), [](const Entry& a, const Entry& b) {
		return a.code != b.code ? a.code < b.code : a.order < b.order;
	});
	out->code_v.clear();
	out->vort_v.clear();
	for (size_t j = 0; j < e.size();) {
		size_t q = j;
		double acc[3] = {0.0, 0.0, 0.0};
		while (q < e.size() && e[q].code == e[j].code) {
			for (int c = 0; c < nc; ++c) acc[c] += double(v[e[q].order * nc + c]);
			++q;
		}
		out->code_v.push_back(e[j].code);
		for (int c = 0; c < nc; ++c) out->vort_v.push_back(float(acc[c]));
		j = q;
	}
	out->code = out->code_v.data();
	out->vort = out->vort_v.data();
	out->n = out->code_v.size();
}

namespace {

// Reference src/redistribution_helper_funcs.cpp:34-85 (histogram search for
// the strength above which about n_desired particles remain).
float strength_threshold(const float* strs, int n, int n_desired) {
	float fmin = n > 0 ? strs[0] : 0.f, fmax = fmin;
	for (int i = 0; i < n; ++i) {
		fmin = fmin < strs[i] ? fmin : strs[i];
		fmax = fmax > strs[i] ? fmax : strs[i];
	}
	double minv = fmin, maxv = fmax, range;
	if (n < n_desired) return float(maxv * 1.05);
	const int ng = 1024;
	const float tol = 0.01f;
	std::vector<float> guess(ng);
	std::vector<int> cnt(ng);
	int k = 0;
	for (;;) {
		range = (maxv - minv) * 1.05;
		for (int i = 0; i < ng; ++i) {
			cnt[i] = 0;
			guess[i] = float(minv + i * range / float(ng - 1));
		}
		for (int i = 0; i < n; ++i) {
			const int b = int(std::floor(double(ng - 1) * (strs[i] - minv) / range));
			if (b < 0) cnt[0]++;
			else if (b >= ng) cnt[ng - 1]++;
			else cnt[b]++;
		}
		int acc = cnt[ng - 1];
		for (int i = ng - 2; i >= 0; --i) {
			maxv = guess[i + 1];
			minv = guess[i];
			acc += cnt[i];
			cnt[i] = acc;
			if (acc > n_desired) { k = i + 1; break; }
		}
		if (minv == maxv || k < 1 || cnt[k] == cnt[k - 1] ||
			std::fabs(float(n_desired - cnt[k]) / float(n_desired)) < double(tol) * 0.6)
			break;
	}
	return guess[k];
}

// dst[0, n) = src[0, n) in parallel chunks (the output can be ~35 MB)
template <class T>
void parallel_copy(T* dst, const T* src, size_t n) {
	const long long chunks = (long long)((n + 65535) / 65536);
#pragma omp parallel for schedule(static)
	for (long long c = 0; c < chunks; ++c) {
		const size_t b = size_t(c) * 65536, e = std::min(n, b + 65536);
		std::memcpy(dst + b, src + b, sizeof(T) * (e - b));
	}
}

float mean_of(const float* s, size_t n) {
	double a = 0.0;
	for (size_t i = 0; i < n; ++i) a += double(s[i]);
	return float(a) / float(n);
}

// Reference src/P3D.cpp:636-662 / src/P2D.cpp:407-432: keep particles with
// strength above `thr` among the first `max_keep`, spread the removed
// vorticity evenly over the kept ones.
template <class P, class AddDeficit>
int remove_weak(P* arr, const float* strs, int n, float thr, int max_keep,
	AddDeficit&& spread)
{
	int j = 0;
	float def[3] = {0.f, 0.f, 0.f};
	for (int i = 0; i < n; ++i) {
		if (strs[i] > thr && i < max_keep) arr[j++] = arr[i];
		else spread(def, arr[i], true);
	}
	for (int c = 0; c < 3; ++c) def[c] = def[c] / float(j);
	for (int i = 0; i < j; ++i) spread(def, arr[i], false);
	return j;
}

void add3(float* def, cvtx_P3D& p, bool collect) {
	for (int c = 0; c < 3; ++c) {
		if (collect) def[c] = p.vorticity.x[c] + def[c];
		else p.vorticity.x[c] = p.vorticity.x[c] + def[c];
	}
}
void add1(float* def, cvtx_P2D& p, bool collect) {
	if (collect) def[0] = p.vorticity + def[0];
	else p.vorticity = p.vorticity + def[0];
}

float norm3(const bsv_V3f& v) {
	return std::sqrt(v.x[0] * v.x[0] + v.x[1] * v.x[1] + v.x[2] * v.x[2]);
}

bool cells_for(int dims, const float* pos, const float* str, int n,
	const cvtx_RedistFunc* f, float gd, RedistGrid* g, RedistCells* cells, const char* what)
{
	if (!redist_grid(dims, pos, n, f, gd, g)) {
		set_error(std::string(what) + ": grid too large for the grid keys");
		return false;
	}
	const int kind = redist_kind(f);
	if (kind >= 0) {
		std::lock_guard<std::recursive_mutex> lk(Runtime::get().lock());
		DeviceContext* ctx = Runtime::get().active_context();
		if (ctx) {
			const cudaError_t e = redist_cells_gpu(*g, kind, pos, str, n, cells, &ctx->redist,
				&ctx->h_redist, ctx->stream);
			if (e != cudaSuccess) {
				cudaGetLastError();
				set_error(std::string(what) + ": " + cudaGetErrorString(e));
				return false;
			}
			return true;
		}
	}
	redist_cells_host(*g, f, pos, str, n, cells);
	return true;
}

}  // namespace
}  // namespace cvtx

using namespace cvtx;

extern "C" {

CVTX_EXPORT int cvtx_P3D_redistribute_on_grid(const cvtx_P3D** in, const int n,
	cvtx_P3D* out, int max_out, const cvtx_RedistFunc* f, float gd, float negligible)
{
	if (n <= 0 || !in || !f || !(gd > 0.f)) return 0;
	std::vector<float> pos(size_t(n) * 3), str(size_t(n) * 3);
#pragma omp parallel for schedule(static)
	for (int i = 0; i < n; ++i)
		for (int c = 0; c < 3; ++c) {
			pos[size_t(i) * 3 + c] = in[i]->coord.x[c];
			str[size_t(i) * 3 + c] = in[i]->vorticity.x[c];
		}
	RedistGrid g;
	RedistCells cells;
	// the GPU path leaves the cells in the device context's pinned buffer:
	// hold the runtime lock until they are decoded
	std::unique_lock<std::recursive_mutex> lk(Runtime::get().lock());
	if (!cells_for(3, pos.data(), str.data(), n, f, gd, &g, &cells,
			"cvtx_P3D_redistribute_on_grid"))
		return 0;
	int m = int(cells.n);
	// default-initialised storage, first touched by the parallel decode
	std::unique_ptr<cvtx_P3D[]> np(new cvtx_P3D[size_t(m > 0 ? m : 1)]);
	std::unique_ptr<float[]> strs(new float[size_t(m > 0 ? m : 1)]);
	const float vol = gd * gd * gd;
#pragma omp parallel for schedule(static)
	for (int i = 0; i < m; ++i) {
		const uint64_t c = cells.code[size_t(i)];
		const uint32_t k[3] = {gather3(c), gather3(c >> 1), gather3(c >> 2)};
		for (int d = 0; d < 3; ++d) {
			np[size_t(i)].coord.x[d] = g.min[d] + gd * float(k[d]);
			np[size_t(i)].vorticity.x[d] = cells.vort[size_t(i) * 3 + d];
		}
		np[size_t(i)].volume = vol;
		strs[size_t(i)] = norm3(np[size_t(i)].vorticity);
	}
	lk.unlock();
	// the mean (FP64, in cell order) and the deficit sums of remove_weak
	// (FP32, in cell order) stay serial: their rounding is part of the result
	const float thr = (m > 0 ? mean_of(strs.get(), size_t(m)) : 0.f) * negligible;
	m = remove_weak(np.get(), strs.get(), m, thr, m, add3);
#pragma omp parallel for schedule(static)
	for (int i = 0; i < m; ++i) strs[size_t(i)] = norm3(np[size_t(i)].vorticity);
	if (out) {
		if (m > max_out) {
			const float t2 = strength_threshold(strs.get(), m, max_out);
			m = remove_weak(np.get(), strs.get(), m, t2, max_out, add3);
		}
		parallel_copy(out, np.get(), size_t(m));
	}
	return m;
}

CVTX_EXPORT int cvtx_P2D_redistribute_on_grid(const cvtx_P2D** in, const int n,
	cvtx_P2D* out, int max_out, const cvtx_RedistFunc* f, float gd, float negligible)
{
	if (n <= 0 || !in || !f || !(gd > 0.f)) return 0;
	std::vector<float> pos(size_t(n) * 2), str(static_cast<size_t>(n));
#pragma omp parallel for schedule(static)
	for (int i = 0; i < n; ++i) {
		pos[size_t(i) * 2] = in[i]->coord.x[0];
		pos[size_t(i) * 2 + 1] = in[i]->coord.x[1];
		str[size_t(i)] = in[i]->vorticity;
	}
	RedistGrid g;
	RedistCells cells;
	std::unique_lock<std::recursive_mutex> lk(Runtime::get().lock());   // as for P3D
	if (!cells_for(2, pos.data(), str.data(), n, f, gd, &g, &cells,
			"cvtx_P2D_redistribute_on_grid"))
		return 0;
	int m = int(cells.n);
	std::unique_ptr<cvtx_P2D[]> np(new cvtx_P2D[size_t(m > 0 ? m : 1)]);
	std::unique_ptr<float[]> strs(new float[size_t(m > 0 ? m : 1)]);
	const float area = gd * gd;
#pragma omp parallel for schedule(static)
	for (int i = 0; i < m; ++i) {
		const uint64_t c = cells.code[size_t(i)];
		np[size_t(i)].coord.x[0] = g.min[0] + gd * float(gather2(c));
		np[size_t(i)].coord.x[1] = g.min[1] + gd * float(gather2(c >> 1));
		np[size_t(i)].vorticity = cells.vort[size_t(i)];
		np[size_t(i)].area = area;
		strs[size_t(i)] = std::fabs(np[size_t(i)].vorticity);
	}
	lk.unlock();
	const float thr = (m > 0 ? mean_of(strs.get(), size_t(m)) : 0.f) * negligible;
	m = remove_weak(np.get(), strs.get(), m, thr, m, add1);
#pragma omp parallel for schedule(static)
	for (int i = 0; i < m; ++i) strs[size_t(i)] = std::fabs(np[size_t(i)].vorticity);
	if (out) {
		if (m > max_out) {
			const float t2 = strength_threshold(strs.get(), m, max_out);
			m = remove_weak(np.get(), strs.get(), m, t2, max_out, add1);
		}
		parallel_copy(out, np.get(), size_t(m));
	}
	return m;
}

}  // extern "C"
