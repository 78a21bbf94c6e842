// sortOT (src/cpu/simplify.cpp:81-93): the two lists of every elected variable in
// CNF_CMP_KEY order (size, first literal, last literal, signature;
// src/cpu/simplify.h:29-42) using the reference's own sort (insertion sort up to
// 20 entries, libstdc++ std::sort above). The lists are first put back into
// clause-store order, the order the reference's lists have when it sorts them,
// so equal keys end up in the reference's relative order.
#pragma once

#include "cnf.cuh"
#include "introsort.cuh"

namespace sigma {

struct KeyLess {
    const Hdr* hdr;
    const u32* lits;
    HD bool operator()(u32 a, u32 b) const {
        const Hdr x = hdr[a], y = hdr[b];
        if (x.size != y.size) return x.size < y.size;
        const u32 x0 = lits[x.start], y0 = lits[y.start];
        if (x0 != y0) return x0 < y0;
        const u32 xb = lits[x.start + x.size - 1], yb = lits[y.start + y.size - 1];
        if (xb != yb) return xb < yb;
        return x.sig < y.sig;
    }
};

struct IdLess {
    HD bool operator()(u32 a, u32 b) const { return a < b; }
};

struct SortArgs {
    Ctx c;
    const u32* pvs;
    u64* ws_bytes;  // kSpreadSlots words summing the elected lists' working set (4*occ + sum(8 + 4*len))
};

// One item per list: 2*k is the positive list of pvs[k], 2*k+1 the negative one.
HD void k_sort_list(const SortArgs& a, u32 k) {
    const u32 l = V2L(a.pvs[k >> 1]) + (k & 1u);
    const u32 n = a.c.ot_size[l];
    u32* d = a.c.ot_refs + a.c.ot_off[l];
    u64 ws = 4ull * n;
    for (u32 i = 0; i < n; i++) ws += 8ull + 4ull * a.c.hdr[d[i]].size;
    spread_sum_add64(a.ws_bytes, ws);
    if (n <= 1) return;
    if (n <= 20) ref_insertion_sort(d, (int)n, IdLess());
    else std_sort_replica(d, d + n, IdLess());
    reference_list_sort(d, (int)n, KeyLess{a.c.hdr, a.c.lits});
}

}  // namespace sigma
