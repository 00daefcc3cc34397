// Packed near groups of the tensor-core kernel sum with one target half.
#include "near_pack.h"

#include <algorithm>
#include <utility>

namespace fmca {

// Packed near groups for the tensor-core kernel sum with one target half:
// the rows of consecutive row leaves back to back in groups of up to cap
// targets, at most two leaves per group.  A group of two leaves
// runs over the union of their source intervals, split into disjoint pieces
// that carry the leaves they serve (imask bit 0: the first leaf, bit 1: the
// second); split[g] = rows of the first leaf.  A leaf joins the group of the
// previous one only if it adds at most half of that leaf's source points
// (the leaves of different clouds of a batched plan have disjoint sources,
// so they never share a group).  false: no packed list (it would not save a
// tenth of the groups, or a check of the result failed).
bool build_near_packed(const Plan& plan, uint32_t cap, PackedNear* out) {
  using Iv = std::pair<uint32_t, uint32_t>;
  const Pattern& P = plan.pat;
  const size_t L = plan.row_leaves.size();
  *out = PackedNear();
  if (L == 0 || cap == 0) return false;
  int64_t unpacked_groups = 0;  // one leaf per group, leaves chunked to cap
  for (size_t l = 0; l < L; ++l)
    unpacked_groups += (plan.rows.size[plan.row_leaves[l]] + cap - 1) / cap;
  struct G {
    uint32_t tbegin, tcount;
    int32_t ivl_begin, ivl_end;
  };
  std::vector<G> groups;
  std::vector<uint32_t> ivl, imask, splits;
  std::vector<std::vector<Iv>> lists(L);
  for (size_t l = 0; l < L; ++l) {
    for (int k = P.near_ptr[l]; k < P.near_ptr[l + 1]; ++k)
      lists[l].push_back({P.near_ivl[2 * k], P.near_ivl[2 * k + 1]});
    std::sort(lists[l].begin(), lists[l].end());
    for (size_t i = 0; i < lists[l].size(); ++i) {  // sorted, disjoint, non-empty
      if (lists[l][i].first >= lists[l][i].second || lists[l][i].second > plan.cols.n)
        return false;
      if (i && lists[l][i].first < lists[l][i - 1].second) return false;
    }
  }
  auto points = [](const std::vector<Iv>& v) {
    uint64_t s = 0;
    for (const Iv& p : v) s += p.second - p.first;
    return s;
  };
  // pieces of the union of a and b with the bits of the lists covering them
  auto merge = [](const std::vector<Iv>& a, const std::vector<Iv>& b, std::vector<Iv>* pcs,
                  std::vector<uint32_t>* bits) {
    std::vector<uint32_t> x;
    for (const Iv& p : a) {
      x.push_back(p.first);
      x.push_back(p.second);
    }
    for (const Iv& p : b) {
      x.push_back(p.first);
      x.push_back(p.second);
    }
    std::sort(x.begin(), x.end());
    x.erase(std::unique(x.begin(), x.end()), x.end());
    size_t ia = 0, ib = 0;
    for (size_t i = 0; i + 1 < x.size(); ++i) {
      const uint32_t x0 = x[i], x1 = x[i + 1];
      while (ia < a.size() && a[ia].second <= x0) ++ia;
      while (ib < b.size() && b[ib].second <= x0) ++ib;
      const uint32_t bt = (ia < a.size() && a[ia].first <= x0 ? 1u : 0u) |
                          (ib < b.size() && b[ib].first <= x0 ? 2u : 0u);
      if (!bt) continue;
      if (!pcs->empty() && pcs->back().second == x0 && bits->back() == bt)
        pcs->back().second = x1;
      else {
        pcs->push_back({x0, x1});
        bits->push_back(bt);
      }
    }
  };
  std::vector<size_t> ord(L);
  for (size_t l = 0; l < L; ++l) ord[l] = l;
  std::sort(ord.begin(), ord.end(), [&](size_t a, size_t b) {
    return plan.rows.begin[plan.row_leaves[a]] < plan.rows.begin[plan.row_leaves[b]];
  });
  // the open group: leaf la from row tb (ra rows), then leaf lb (rb rows)
  size_t la = 0, lb = 0;
  uint32_t tb = 0, ra = 0, rb = 0;
  int nseg = 0;
  auto flush = [&]() {
    if (!nseg) return;
    const int ib = (int)(ivl.size() / 2);
    std::vector<Iv> pcs;
    std::vector<uint32_t> bits;
    if (nseg == 1) {
      pcs = lists[la];
      bits.assign(pcs.size(), 1u);
    } else {
      merge(lists[la], lists[lb], &pcs, &bits);
    }
    for (size_t i = 0; i < pcs.size(); ++i) {
      ivl.push_back(pcs[i].first);
      ivl.push_back(pcs[i].second);
      imask.push_back(bits[i]);
    }
    groups.push_back(G{tb, ra + rb, ib, (int32_t)(ivl.size() / 2)});
    splits.push_back(ra);
    nseg = 0;
    ra = rb = 0;
  };
  for (size_t oi = 0; oi < L; ++oi) {
    const size_t l = ord[oi];
    const int c = plan.row_leaves[l];
    uint32_t row = plan.rows.begin[c], left = plan.rows.size[c];
    while (left > 0) {
      if (nseg == 1) {  // join the open group, or close it
        std::vector<Iv> pcs;
        std::vector<uint32_t> bits;
        merge(lists[la], lists[l], &pcs, &bits);
        uint64_t added = 0;
        for (size_t i = 0; i < pcs.size(); ++i)
          if (bits[i] == 2u) added += pcs[i].second - pcs[i].first;
        if (2 * added > points(lists[la])) flush();
      } else if (nseg == 2) {
        flush();
      }
      const uint32_t take = std::min(left, cap - (ra + rb));
      if (nseg == 0) {
        la = l;
        tb = row;
        ra = take;
        nseg = 1;
      } else {
        lb = l;
        rb = take;
        nseg = 2;
      }
      row += take;
      left -= take;
      if (ra + rb == cap) flush();
    }
  }
  flush();
  if ((int64_t)groups.size() * 10 > unpacked_groups * 9) return false;
  // checks: the groups hold as many rows as the leaves, at most cap each;
  // every group's pieces sorted, disjoint and inside the columns, flags 1..3
  // (1 only in groups of one leaf)
  uint64_t rows = 0;
  for (size_t l = 0; l < L; ++l) rows += plan.rows.size[plan.row_leaves[l]];
  uint64_t seen = 0;
  for (size_t g = 0; g < groups.size(); ++g) {
    const G& gr = groups[g];
    if (gr.tcount == 0 || gr.tcount > cap || splits[g] == 0 || splits[g] > gr.tcount ||
        gr.ivl_begin > gr.ivl_end)
      return false;
    uint32_t prev = 0;
    for (int k = gr.ivl_begin; k < gr.ivl_end; ++k) {
      const uint32_t b = ivl[2 * k], e = ivl[2 * k + 1], m = imask[k];
      if (b >= e || e > plan.cols.n || (k > gr.ivl_begin && b < prev) || m == 0u || m > 3u ||
          (splits[g] == gr.tcount && m != 1u))
        return false;
      prev = e;
    }
    seen += gr.tcount;
  }
  if (seen != rows) return false;
  // most work first, split permuted alongside
  std::vector<uint64_t> work(groups.size());
  for (size_t i = 0; i < groups.size(); ++i) {
    uint64_t s = 0;
    for (int k = groups[i].ivl_begin; k < groups[i].ivl_end; ++k) s += ivl[2 * k + 1] - ivl[2 * k];
    work[i] = s;
  }
  std::vector<size_t> order(groups.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(),
                   [&](size_t a, size_t b) { return work[a] > work[b]; });
  for (size_t i : order) {
    out->tbegin.push_back(groups[i].tbegin);
    out->tcount.push_back(groups[i].tcount);
    out->ivl_begin.push_back(groups[i].ivl_begin);
    out->ivl_end.push_back(groups[i].ivl_end);
    out->split.push_back(splits[i]);
  }
  out->ivl.swap(ivl);
  out->imask.swap(imask);
  return true;
}

}  // namespace fmca
