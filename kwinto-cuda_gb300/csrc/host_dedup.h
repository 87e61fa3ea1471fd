// host_dedup.h -- host-side deduplication of a portfolio into PDEs, and the radix
// sort that orders the PDEs of an uneven batch into tiles and buckets.
//
// The key is the reference's (src/Pricer/kwFd1d.cpp:28-65): options that share
// (t, r, q, z, e, w) -- plus (x_dim, t_dim) for uneven batches, where the reference
// would need one init per shape -- are one PDE.  The reference sorts the options
// by that key (O(n log n)); an open-addressing hash table finds the same groups in
// O(n).  PDEs are numbered in order of their first option.  Keys compare by value
// as in the reference's ordering (+0 == -0); a NaN field matches nothing, so such an
// option keeps its own PDE and is reported as bad input instead of taking a
// neighbour's price.
#pragma once

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <utility>
#include <vector>

#include "kwg.h"

namespace kwg {

inline uint64_t key_bits(double v)
{
    uint64_t b;
    std::memcpy(&b, &v, sizeof b);
    return v == 0. ? 0ull : b;  // +0 and -0 hash alike
}

inline uint64_t host_key_hash(const kwg_option& o, int32_t x_dim, int32_t t_dim)
{
    uint64_t h = 0x9E3779B97F4A7C15ull;
    for (double v : {o.t, o.r, o.q, o.z}) {
        h = (h ^ key_bits(v)) * 0xBF58476D1CE4E5B9ull;
        h ^= h >> 31;
    }
    h = (h ^ ((uint64_t)o.e << 8 | (uint8_t)o.w) ^ ((uint64_t)(uint32_t)x_dim << 16) ^
         ((uint64_t)(uint32_t)t_dim << 40)) *
        0x94D049BB133111EBull;
    return h ^ (h >> 29);
}

// Fills asset2pde (n entries) and pde2asset (the first option of each distinct key)
// and returns the number of PDEs.  x_dims, t_dims: per-option grid shape of an
// uneven batch, or nullptr.
inline size_t dedup_host(const kwg_option* opts, size_t n, const int32_t* x_dims, const int32_t* t_dims,
                         std::vector<int32_t>& asset2pde, std::vector<uint32_t>& pde2asset)
{
    size_t cap = 16;
    while (cap < 2 * n) cap <<= 1;
    const size_t mask = cap - 1;
    std::vector<int32_t> table(cap, -1);
    asset2pde.resize(n);
    pde2asset.clear();
    pde2asset.reserve(n);
    for (size_t i = 0; i < n; ++i) {
        const kwg_option& o = opts[i];
        const int32_t xi = x_dims ? x_dims[i] : 0, ti = t_dims ? t_dims[i] : 0;
        size_t h = host_key_hash(o, xi, ti) & mask;
        for (;;) {
            const int32_t p = table[h];
            if (p < 0) {
                table[h] = (int32_t)pde2asset.size();
                asset2pde[i] = table[h];
                pde2asset.push_back((uint32_t)i);
                break;
            }
            const uint32_t a = pde2asset[p];
            const kwg_option& b = opts[a];
            if (o.t == b.t && o.r == b.r && o.q == b.q && o.z == b.z && o.e == b.e && o.w == b.w &&
                (!x_dims || x_dims[a] == xi) && (!t_dims || t_dims[a] == ti)) {
                asset2pde[i] = p;
                break;
            }
            h = (h + 1) & mask;
        }
    }
    return pde2asset.size();
}

// Stable LSD radix sort of (key, index) pairs by key, 16 bits per pass; a pass
// whose digit is the same for every key is skipped (layout keys vary in few bits).
// Equal keys keep their order, so pairs built in index order come out as
// std::sort would order them.
inline void radix_sort_pairs(std::vector<std::pair<uint64_t, uint32_t>>& kv)
{
    const size_t m = kv.size();
    if (m < 2) return;
    uint64_t all_or = 0, all_and = ~0ull;
    for (const auto& e : kv) {
        all_or |= e.first;
        all_and &= e.first;
    }
    const uint64_t varying = all_or ^ all_and;
    std::vector<std::pair<uint64_t, uint32_t>> tmp(m);
    std::vector<uint32_t> cnt(1u << 16);
    for (int shift = 0; shift < 64; shift += 16) {
        if (((varying >> shift) & 0xffffu) == 0) continue;
        std::fill(cnt.begin(), cnt.end(), 0u);
        for (const auto& e : kv) ++cnt[(e.first >> shift) & 0xffffu];
        uint32_t sum = 0;
        for (uint32_t& c : cnt) {
            const uint32_t v = c;
            c = sum;
            sum += v;
        }
        for (const auto& e : kv) tmp[cnt[(e.first >> shift) & 0xffffu]++] = e;
        kv.swap(tmp);
    }
}

}  // namespace kwg
