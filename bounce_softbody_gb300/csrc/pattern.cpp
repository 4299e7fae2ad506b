// Host-side construction of a body's block pattern and of the precomputed scatter maps.
//
// The reference accumulates every element block into linked-list rows with a linear search
// per insertion (include/bounce_softbody/sparse/sparse_mat33.h:268-288). Here the pattern is
// built once per topology: each row lists its diagonal first, then its other columns in
// increasing order; every (element, local row a, local column b) contribution is assigned its
// slot ahead of time and the contributions of a slot are listed in element order. Assembly then
// gathers per slot in that fixed order, which makes it deterministic (bitwise reproducible)
// without float atomics.
#include "internal.h"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

namespace b3g {

namespace {

struct Inc
{
	uint32_t kind;  // 0 tet, 1 tri, 2 spring, 3 stretch/shear triangle, 4 mouse spring
	uint32_t e;
	uint32_t a;     // local index of the row vertex in the element
};

template <class T>
T* dup(const std::vector<T>& v)
{
	T* p = (T*)std::malloc(std::max<size_t>(1, v.size()) * sizeof(T));
	if (!v.empty()) std::memcpy(p, v.data(), v.size() * sizeof(T));
	return p;
}

} // namespace

// Re-lays a CSR list (ptr over `items` items) so that the items of each group of 32 consecutive
// items interleave their entries: entry t of item j goes to start[j] + 32 t. Padding entries
// (for items shorter than the longest of their group) are zero and never read.
static bool interleave(const std::vector<uint32_t>& ptr, const std::vector<uint32_t>& list, size_t items,
                       Pattern::Lists* out, char* err, size_t errlen)
{
	std::vector<uint32_t> start(items, 0);
	std::vector<uint16_t> cnt(items, 0);
	uint64_t cursor = 0;
	for (size_t g = 0; g < items; g += kSlice)
	{
		uint32_t m = 0;
		for (size_t j = g; j < g + kSlice && j < items; ++j) m = std::max(m, ptr[j + 1] - ptr[j]);
		if (m > 65535)
		{
			std::snprintf(err, errlen, "an item has %u contributions (limit 65535)", m);
			return false;
		}
		for (size_t j = g; j < g + kSlice && j < items; ++j)
		{
			start[j] = (uint32_t)(cursor + (j - g));
			cnt[j] = (uint16_t)(ptr[j + 1] - ptr[j]);
		}
		cursor += (uint64_t)kSlice * m;
		if (cursor >= (1ull << 32))
		{
			std::snprintf(err, errlen, "contribution lists exceed 2^32 entries");
			return false;
		}
	}
	std::vector<uint32_t> il(std::max<uint64_t>(cursor, 1), 0u);
	for (size_t j = 0; j < items; ++j)
		for (uint32_t t = 0; t < cnt[j]; ++t) il[start[j] + (size_t)kSlice * t] = list[ptr[j] + t];
	out->start = (uint32_t*)std::malloc(std::max<size_t>(items, 1) * sizeof(uint32_t));
	out->cnt = (uint16_t*)std::malloc(std::max<size_t>(items, 1) * sizeof(uint16_t));
	out->list = (uint32_t*)std::malloc(il.size() * sizeof(uint32_t));
	if (items)
	{
		std::memcpy(out->start, start.data(), items * sizeof(uint32_t));
		std::memcpy(out->cnt, cnt.data(), items * sizeof(uint16_t));
	}
	std::memcpy(out->list, il.data(), il.size() * sizeof(uint32_t));
	out->len = il.size();
	out->items = items;
	return true;
}

static void free_lists(Pattern::Lists* l)
{
	std::free(l->start);
	std::free(l->cnt);
	std::free(l->list);
	*l = Pattern::Lists();
}

std::vector<uint32_t> tet_storage_order(uint32_t nt, const uint32_t* tets)
{
	std::vector<uint32_t> order(nt);
	for (uint32_t e = 0; e < nt; ++e) order[e] = e;
	// signatures as offsets from the first vertex; a mesh with more than kMaxSignatures of them
	// has no repeating cell to exploit
	constexpr size_t kMaxSignatures = 64;
	struct Sig
	{
		int64_t d[3];
		bool operator<(const Sig& o) const
		{
			return d[0] != o.d[0] ? d[0] < o.d[0] : (d[1] != o.d[1] ? d[1] < o.d[1] : d[2] < o.d[2]);
		}
		bool operator==(const Sig& o) const { return d[0] == o.d[0] && d[1] == o.d[1] && d[2] == o.d[2]; }
	};
	auto sig_of = [&](uint32_t e) {
		const uint32_t* t = tets + 4 * (size_t)e;
		return Sig{{(int64_t)t[1] - t[0], (int64_t)t[2] - t[0], (int64_t)t[3] - t[0]}};
	};
	std::vector<Sig> seen;
	for (uint32_t e = 0; e < nt; ++e)
	{
		const Sig s = sig_of(e);
		if (std::find(seen.begin(), seen.end(), s) != seen.end()) continue;
		if (seen.size() == kMaxSignatures) return order;
		seen.push_back(s);
	}
	std::sort(seen.begin(), seen.end());
	std::vector<uint32_t> group(nt);
	for (uint32_t e = 0; e < nt; ++e)
		group[e] = (uint32_t)(std::lower_bound(seen.begin(), seen.end(), sig_of(e)) - seen.begin());
	std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
		if (group[a] != group[b]) return group[a] < group[b];
		return tets[4 * (size_t)a] < tets[4 * (size_t)b];
	});
	return order;
}

void free_pattern(Pattern* p)
{
	std::free(p->slice_ptr);
	std::free(p->col);
	std::free(p->rowlen);
	free_lists(&p->tet);
	free_lists(&p->blk);
	free_lists(&p->vt);
	free_lists(&p->vb);
	*p = Pattern();
}

bool build_pattern(uint32_t n, uint32_t nt, const uint32_t* tets, uint32_t ntr, const uint32_t* tris,
                   uint32_t ns, const uint32_t* springs, uint32_t nbw, const uint32_t* bw, uint32_t nms,
                   const uint32_t* ms, const uint32_t* tet_rank, Pattern* out, char* err, size_t errlen)
{
	*out = Pattern();
	if (n == 0)
	{
		std::snprintf(err, errlen, "body has no vertices");
		return false;
	}
	if ((uint64_t)nt >= (1ull << 28))
	{
		std::snprintf(err, errlen, "too many tetrahedra (%u, limit 2^28)", nt);
		return false;
	}

	// incidence lists, vertex-major, elements in increasing order per kind
	std::vector<uint32_t> inc_cnt(n + 1, 0);
	auto check = [&](uint32_t id, const char* what, uint32_t e) -> bool {
		if (id >= n)
		{
			std::snprintf(err, errlen, "%s %u references vertex %u >= vertex_count %u", what, e, id, n);
			return false;
		}
		return true;
	};
	for (uint32_t e = 0; e < nt; ++e)
		for (int a = 0; a < 4; ++a)
		{
			if (!check(tets[4 * e + a], "tetrahedron", e)) return false;
			for (int b = 0; b < a; ++b)
				if (tets[4 * e + a] == tets[4 * e + b])
				{
					std::snprintf(err, errlen, "tetrahedron %u repeats vertex %u", e, tets[4 * e + a]);
					return false;
				}
			inc_cnt[tets[4 * e + a] + 1]++;
		}
	for (uint32_t e = 0; e < ntr; ++e)
		for (int a = 0; a < 3; ++a)
		{
			if (!check(tris[3 * e + a], "triangle", e)) return false;
			for (int b = 0; b < a; ++b)
				if (tris[3 * e + a] == tris[3 * e + b])
				{
					std::snprintf(err, errlen, "triangle %u repeats vertex %u", e, tris[3 * e + a]);
					return false;
				}
			inc_cnt[tris[3 * e + a] + 1]++;
		}
	for (uint32_t e = 0; e < ns; ++e)
		for (int a = 0; a < 2; ++a)
		{
			if (!check(springs[2 * e + a], "spring", e)) return false;
			inc_cnt[springs[2 * e + a] + 1]++;
		}
	for (uint32_t e = 0; e < nbw; ++e)
		for (int a = 0; a < 3; ++a)
		{
			if (!check(bw[3 * e + a], "stretch/shear triangle", e)) return false;
			for (int b = 0; b < a; ++b)
				if (bw[3 * e + a] == bw[3 * e + b])
				{
					std::snprintf(err, errlen, "stretch/shear triangle %u repeats vertex %u", e, bw[3 * e + a]);
					return false;
				}
			inc_cnt[bw[3 * e + a] + 1]++;
		}
	// a mouse spring may name a vertex twice (weights of a degenerate triangle): each local
	// index is its own incidence and the slot lists sum both, as the reference's dfdx(i, j) += does
	for (uint32_t e = 0; e < nms; ++e)
		for (int a = 0; a < 4; ++a)
		{
			if (!check(ms[4 * e + a], "mouse spring", e)) return false;
			inc_cnt[ms[4 * e + a] + 1]++;
		}
	for (uint32_t i = 0; i < n; ++i) inc_cnt[i + 1] += inc_cnt[i];
	std::vector<Inc> inc(inc_cnt[n]);
	{
		std::vector<uint32_t> fill(inc_cnt.begin(), inc_cnt.end() - 1);
		for (uint32_t e = 0; e < nt; ++e)
			for (uint32_t a = 0; a < 4; ++a) inc[fill[tets[4 * e + a]]++] = Inc{0, e, a};
		for (uint32_t e = 0; e < ntr; ++e)
			for (uint32_t a = 0; a < 3; ++a) inc[fill[tris[3 * e + a]]++] = Inc{1, e, a};
		for (uint32_t e = 0; e < ns; ++e)
			for (uint32_t a = 0; a < 2; ++a) inc[fill[springs[2 * e + a]]++] = Inc{2, e, a};
		for (uint32_t e = 0; e < nbw; ++e)
			for (uint32_t a = 0; a < 3; ++a) inc[fill[bw[3 * e + a]]++] = Inc{3, e, a};
		for (uint32_t e = 0; e < nms; ++e)
			for (uint32_t a = 0; a < 4; ++a) inc[fill[ms[4 * e + a]]++] = Inc{4, e, a};
	}

	auto elem_vertex = [&](const Inc& c, uint32_t b) -> uint32_t {
		if (c.kind == 0) return tets[4 * c.e + b];
		if (c.kind == 1) return tris[3 * c.e + b];
		if (c.kind == 2) return springs[2 * c.e + b];
		if (c.kind == 3) return bw[3 * c.e + b];
		return ms[4 * c.e + b];
	};
	auto elem_size = [](uint32_t kind) -> uint32_t {
		static const uint32_t size[5] = {4u, 3u, 2u, 3u, 4u};
		return size[kind];
	};
	// first block and first vector of each explicit kind
	const uint64_t blk_bw = 9ull * ntr + ns, blk_ms = blk_bw + 9ull * nbw, blk_end = blk_ms + 16ull * nms;
	const uint64_t vec_bw = 3ull * ntr + ns, vec_ms = vec_bw + 3ull * nbw;
	if (blk_end >= (1ull << 31))
	{
		std::snprintf(err, errlen, "explicit blocks exceed 2^31");
		return false;
	}

	// rows: diagonal first, then the other columns ascending
	std::vector<uint32_t> rowptr(n + 1, 0);
	std::vector<uint32_t> cols;
	cols.reserve((size_t)n * 16);
	std::vector<uint32_t> tmp;
	for (uint32_t i = 0; i < n; ++i)
	{
		tmp.clear();
		for (uint32_t k = inc_cnt[i]; k < inc_cnt[i + 1]; ++k)
			for (uint32_t b = 0; b < elem_size(inc[k].kind); ++b)
			{
				uint32_t j = elem_vertex(inc[k], b);
				if (j != i) tmp.push_back(j);
			}
		std::sort(tmp.begin(), tmp.end());
		tmp.erase(std::unique(tmp.begin(), tmp.end()), tmp.end());
		if (tmp.size() + 1 > 255)
		{
			std::snprintf(err, errlen, "vertex %u has %zu neighbours (limit 254)", i, tmp.size());
			return false;
		}
		cols.push_back(i);
		cols.insert(cols.end(), tmp.begin(), tmp.end());
		rowptr[i + 1] = (uint32_t)cols.size();
	}
	auto find_k = [&](uint32_t i, uint32_t j) -> uint32_t {
		if (j == i) return 0;
		uint32_t lo = rowptr[i] + 1, hi = rowptr[i + 1];
		while (lo < hi)
		{
			uint32_t mid = (lo + hi) >> 1;
			if (cols[mid] < j) lo = mid + 1;
			else hi = mid;
		}
		return lo - rowptr[i];
	};

	// SELL-32 slots
	Pattern P;
	P.n = (int)n;
	P.nslices = (int)((n + kSlice - 1) / kSlice);
	P.npad = P.nslices * kSlice;
	P.nnzb = cols.size();
	std::vector<int> slice_ptr(P.nslices + 1, 0);
	std::vector<uint8_t> rowlen(P.npad, 0);
	for (uint32_t i = 0; i < n; ++i) rowlen[i] = (uint8_t)(rowptr[i + 1] - rowptr[i]);
	for (int s = 0; s < P.nslices; ++s)
	{
		int w = 0;
		for (int l = 0; l < kSlice; ++l) w = std::max(w, (int)rowlen[s * kSlice + l]);
		w = (w + kGroup - 1) / kGroup * kGroup;  // whole groups of kGroup slots
		P.maxw = std::max(P.maxw, w);
		slice_ptr[s + 1] = slice_ptr[s] + w * kSlice;
	}
	P.nslots = slice_ptr[P.nslices];
	// contribution-list item of (row i, k-th block): list_item(s, k, lane) = slice_ptr[s] + 32 k + lane
	auto slot_of = [&](uint32_t i, uint32_t k) -> uint32_t {
		return (uint32_t)slice_ptr[i / kSlice] + k * kSlice + (i % kSlice);
	};
	// block slots: block_slot(s, k, lane) = slice_ptr[s] + 128 (k / 4) + 4 lane + k % 4
	std::vector<int> col(P.nslots, 0);
	for (int s = 0; s < P.nslices; ++s)
		for (int l = 0; l < kSlice; ++l)
		{
			uint32_t i = (uint32_t)(s * kSlice + l);
			int w = (slice_ptr[s + 1] - slice_ptr[s]) / kSlice;
			for (int k = 0; k < w; ++k)
				col[block_slot(slice_ptr[s], k, l)] =
				    (i < n && (uint32_t)k < rowlen[i]) ? (int)cols[rowptr[i] + k] : (int)std::min<uint32_t>(i, n - 1);
		}

	// contribution counts per slot
	std::vector<uint32_t> tcnt(P.nslots + 1, 0), bcnt(P.nslots + 1, 0);
	for (uint32_t i = 0; i < n; ++i)
		for (uint32_t k = inc_cnt[i]; k < inc_cnt[i + 1]; ++k)
		{
			const Inc& c = inc[k];
			for (uint32_t b = 0; b < elem_size(c.kind); ++b)
			{
				uint32_t slot = slot_of(i, find_k(i, elem_vertex(c, b)));
				if (c.kind == 0) tcnt[slot + 1]++;
				else bcnt[slot + 1]++;
			}
		}
	for (int s = 0; s < P.nslots; ++s)
	{
		tcnt[s + 1] += tcnt[s];
		bcnt[s + 1] += bcnt[s];
	}
	std::vector<uint32_t> tlist(tcnt[P.nslots]), blist(bcnt[P.nslots]);
	{
		std::vector<uint32_t> tf(tcnt.begin(), tcnt.end() - 1), bf(bcnt.begin(), bcnt.end() - 1);
		// rows in order, incidences in element order: each slot's list comes out sorted by element
		for (uint32_t i = 0; i < n; ++i)
			for (uint32_t k = inc_cnt[i]; k < inc_cnt[i + 1]; ++k)
			{
				const Inc& c = inc[k];
				for (uint32_t b = 0; b < elem_size(c.kind); ++b)
				{
					uint32_t slot = slot_of(i, find_k(i, elem_vertex(c, b)));
					if (c.kind == 0) tlist[tf[slot]++] = ((tet_rank ? tet_rank[c.e] : c.e) << 4) | (c.a << 2) | b;
					else if (c.kind == 1) blist[bf[slot]++] = ((9u * c.e + 3u * c.a + b) << 1);
					else if (c.kind == 2) blist[bf[slot]++] = ((9u * ntr + c.e) << 1) | (c.a != b ? 1u : 0u);
					else if (c.kind == 3) blist[bf[slot]++] = (uint32_t)(blk_bw + 9u * c.e + 3u * c.a + b) << 1;
					else blist[bf[slot]++] = (uint32_t)(blk_ms + 16u * c.e + 4u * c.a + b) << 1;
				}
			}
	}

	// vertex lists of right-hand-side contributions
	std::vector<uint32_t> vtp(P.npad + 1, 0), vbp(P.npad + 1, 0), vtl, vbl;
	vtl.reserve(4 * (size_t)nt);
	vbl.reserve(3 * (size_t)ntr + 2 * (size_t)ns + 3 * (size_t)nbw + 4 * (size_t)nms);
	for (uint32_t i = 0; i < n; ++i)
	{
		for (uint32_t k = inc_cnt[i]; k < inc_cnt[i + 1]; ++k)
		{
			const Inc& c = inc[k];
			if (c.kind == 0) vtl.push_back(((tet_rank ? tet_rank[c.e] : c.e) << 2) | c.a);
			else if (c.kind == 1) vbl.push_back((3u * c.e + c.a) << 1);
			else if (c.kind == 2) vbl.push_back(((3u * ntr + c.e) << 1) | (c.a == 1 ? 1u : 0u));
			else if (c.kind == 3) vbl.push_back((uint32_t)(vec_bw + 3u * c.e + c.a) << 1);
			else vbl.push_back((uint32_t)(vec_ms + 4u * c.e + c.a) << 1);
		}
		vtp[i + 1] = (uint32_t)vtl.size();
		vbp[i + 1] = (uint32_t)vbl.size();
	}
	for (int i = (int)n; i < P.npad; ++i)
	{
		vtp[i + 1] = vtp[i];
		vbp[i + 1] = vbp[i];
	}

	if (!interleave(tcnt, tlist, P.nslots, &P.tet, err, errlen) || !interleave(bcnt, blist, P.nslots, &P.blk, err, errlen) ||
	    !interleave(vtp, vtl, P.npad, &P.vt, err, errlen) || !interleave(vbp, vbl, P.npad, &P.vb, err, errlen))
	{
		free_pattern(&P);
		return false;
	}
	P.slice_ptr = dup(slice_ptr);
	P.col = dup(col);
	P.rowlen = dup(rowlen);
	*out = P;
	return true;
}

} // namespace b3g
