// Host-side construction of the CSR pattern, the element->CSR slot map and
// the element-chunk reduction plan (see tm_chunk_plan in the public header).
//
// Pattern and slot map reproduce ElementAssembler.from_mesh
// (assemble/element_assembler.py:811-830): every local pair (i, j) of every
// element contributes (conn[e,i], conn[e,j]); the pattern is the set of
// distinct pairs sorted row-major, stored as int32 rows/cols, and the slot
// map gives, element-major then i then j, the position of each pair in that
// list.  Here it is built by a counting sort on rows and a per-row sort, in
// O(E*B^2 log(deg)) time, instead of SciPy's COO->CSR conversion.
#include "../../include/tensormesh_gb300.h"
#include "tm_status.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>
#include <numeric>
#include <thread>
#include <type_traits>
#include <utility>
#include <vector>

// Allocator whose value-less construct leaves an element uninitialised:
// resize() then does not zero the pages on one thread, and the parallel
// loops that fill the arrays are the first to touch them.
template <class T>
struct uninit_alloc : std::allocator<T> {
    using value_type = T;
    template <class U>
    struct rebind {
        using other = uninit_alloc<U>;
    };
    uninit_alloc() = default;
    template <class U>
    uninit_alloc(const uninit_alloc<U>&) noexcept {}
    template <class U>
    void construct(U* q) noexcept(std::is_nothrow_default_constructible<U>::value) {
        ::new ((void*)q) U;
    }
    template <class U, class... A>
    void construct(U* q, A&&... a) {
        ::new ((void*)q) U(std::forward<A>(a)...);
    }
};
template <class T>
using buffer = std::vector<T, uninit_alloc<T>>;

struct tm_host_plan {
    int32_t kind = 0, n_basis = 0, n_local = 0, chunk_elems = 0, n_chunks = 0;
    int64_t n_elements = 0, n_points = 0, nnz = 0, n_partials = 0;
    buffer<int32_t> edge_row, edge_col;
    buffer<int64_t> slot;
    buffer<int32_t> chunk_begin, chunk_contrib, slot_ptr, slot_target, slot_mirror;
    int32_t max_chunk_slots = 0, max_chunk_contrib = 0;
    buffer<uint16_t> contrib;
    buffer<int32_t> shared_ptr, shared_target, shared_mirror;
    buffer<int32_t> conn, perm;
};

namespace {

struct Contribution {
    int32_t target;
    int32_t mirror;
    uint16_t code;
};

// host threads for plan construction: TM_HOST_THREADS if set, else all
// hardware threads (at most 64)
int host_threads() {
    const char* env = std::getenv("TM_HOST_THREADS");
    int n = env ? std::atoi(env) : 0;
    if (n <= 0) n = (int)std::thread::hardware_concurrency();
    return std::max(1, std::min(n, 64));
}

// items per thread below which a loop of simple per-item work stays on fewer
// threads (starting a thread costs tens of microseconds)
constexpr int64_t kGrain = 1 << 15;

// host threads for n items of at least `grain` items each
int threads_for(int64_t n, int64_t grain) {
    return (int)std::max<int64_t>(1, std::min<int64_t>(host_threads(), n / grain));
}

// f(begin, end) over at most T contiguous ranges of [0, n), of `grain` items
// at least, on as many threads (the calling thread takes the first, and the
// ranges of threads that could not be started); an allocation failure on
// any thread is rethrown as bad_alloc
template <class F>
void parallel_for(int64_t n, int T, F&& f, int64_t grain = 1) {
    if (n <= 0) return;
    T = (int)std::min<int64_t>(T, std::max<int64_t>(1, n / std::max<int64_t>(1, grain)));
    if (T <= 1) {
        f(int64_t(0), n);
        return;
    }
    const int64_t step = (n + T - 1) / T;
    std::atomic<bool> failed(false);
    auto run = [&](int64_t b, int64_t e) {
        try {
            f(b, e);
        } catch (...) {
            failed = true;
        }
    };
    std::vector<std::thread> pool;
    int64_t rest = std::min(n, step);   // [rest, n) has no thread: the calling thread runs it
    try {
        pool.reserve(T - 1);
        for (int t = 1; t < T; ++t) {
            const int64_t b = t * step, e = std::min(n, b + step);
            if (b >= e) break;
            pool.emplace_back(run, b, e);
            rest = e;
        }
    } catch (...) {
    }
    run(0, std::min(n, step));
    if (rest < n) run(rest, n);
    for (auto& th : pool) th.join();
    if (failed) throw std::bad_alloc();
}

void build_pattern(tm_host_plan& p, const int64_t* conn) {
    const int64_t E = p.n_elements, N = p.n_points;
    const int B = p.n_basis;
    // counting sort of all E*B*B (row, col) pairs by row: contiguous element
    // ranges count their rows, then each range fills its rows after the
    // earlier ranges' entries (the sequential order), on host threads
    const int T = threads_for(E, kGrain / 4);
    const int64_t estep = (E + T - 1) / T;
    std::vector<std::vector<int32_t>> cnt(T, std::vector<int32_t>(N, 0));
    parallel_for(T, T, [&](int64_t t0, int64_t t1) {
        for (int64_t t = t0; t < t1; ++t)
            for (int64_t e = t * estep; e < std::min(E, (t + 1) * estep); ++e)
                for (int a = 0; a < B; ++a) cnt[t][conn[e * B + a]] += B;
    });
    std::vector<int64_t> row_ptr(N + 1, 0);
    for (int64_t r = 0; r < N; ++r) {
        int64_t o = 0;
        for (int t = 0; t < T; ++t) {
            const int32_t c = cnt[t][r];
            cnt[t][r] = (int32_t)o;   // offset of range t within row r
            o += c;
        }
        row_ptr[r + 1] = row_ptr[r] + o;
    }
    buffer<int32_t> cols(row_ptr[N]);
    parallel_for(T, T, [&](int64_t t0, int64_t t1) {
        for (int64_t t = t0; t < t1; ++t)
            for (int64_t e = t * estep; e < std::min(E, (t + 1) * estep); ++e)
                for (int a = 0; a < B; ++a) {
                    const int64_t r = conn[e * B + a];
                    int32_t& f = cnt[t][r];
                    for (int b = 0; b < B; ++b) cols[row_ptr[r] + f++] = (int32_t)conn[e * B + b];
                }
    });
    cnt.clear();
    cnt.shrink_to_fit();
    // sort + unique per row, then compaction (rows on host threads)
    const int TR = host_threads();
    std::vector<int64_t> ucnt(N, 0);
    parallel_for(N, TR, [&](int64_t r0, int64_t r1) {
        for (int64_t r = r0; r < r1; ++r) {
            int32_t* s = cols.data() + row_ptr[r];
            int32_t* t = cols.data() + row_ptr[r + 1];
            std::sort(s, t);
            ucnt[r] = std::unique(s, t) - s;
        }
    }, kGrain / 16);
    std::vector<int64_t> urow_ptr(N + 1, 0);
    for (int64_t r = 0; r < N; ++r) urow_ptr[r + 1] = urow_ptr[r] + ucnt[r];
    const int64_t nnz = urow_ptr[N];
    p.nnz = nnz;
    p.edge_row.resize(nnz);
    p.edge_col.resize(nnz);
    parallel_for(N, TR, [&](int64_t r0, int64_t r1) {
        for (int64_t r = r0; r < r1; ++r) {
            std::copy(cols.begin() + row_ptr[r], cols.begin() + row_ptr[r] + ucnt[r], p.edge_col.begin() + urow_ptr[r]);
            std::fill(p.edge_row.begin() + urow_ptr[r], p.edge_row.begin() + urow_ptr[r + 1], (int32_t)r);
        }
    }, kGrain);
    // slot map, element-major, i-major, j-minor
    p.slot.resize((size_t)E * B * B);
    const int32_t* ucol = p.edge_col.data();
    parallel_for(E, TR, [&](int64_t e0, int64_t e1) {
        for (int64_t e = e0; e < e1; ++e)
            for (int a = 0; a < B; ++a) {
                const int64_t r = conn[e * B + a];
                const int32_t* s = ucol + urow_ptr[r];
                const int32_t* t = ucol + urow_ptr[r + 1];
                for (int b = 0; b < B; ++b) {
                    const int32_t c = (int32_t)conn[e * B + b];
                    p.slot[(e * B + a) * B + b] = (int64_t)(std::lower_bound(s, t, c) - ucol);
                }
            }
    }, kGrain / 8);
}

int build_chunks(tm_host_plan& p) {
    const int64_t E = p.n_elements;
    const int B = p.n_basis, NL = p.n_local, CH = p.chunk_elems;
    const bool matrix = p.kind == TM_PLAN_KIND_MATRIX;
    const int64_t n_targets = matrix ? p.nnz : p.n_points;
    if ((int64_t)CH * NL * 2 > 65536) return TM_ERR_TOO_LARGE;
    p.n_chunks = (int32_t)((E + CH - 1) / CH);
    // Chunks are independent: ranges of chunks are built on host threads
    // into per-range arrays, then concatenated in chunk order, so the plan
    // does not depend on the number of threads.
    struct Part {
        std::vector<int32_t> slot_target, slot_mirror, slot_len, chunk_slots;
        std::vector<uint16_t> contrib;
    };
    const int T = host_threads();
    const int TP = (int)std::max<int64_t>(1, std::min<int64_t>(T, p.n_chunks / 16));   // 16 chunks a thread at least
    const int64_t per = std::max<int64_t>(1, (p.n_chunks + TP - 1) / TP);
    const int n_parts = (int)((p.n_chunks + per - 1) / per);
    std::vector<Part> parts(n_parts);
    parallel_for(n_parts, TP, [&](int64_t part_begin, int64_t part_end) {
        // A chunk holds fewer than 65536 contributions (codes are 16-bit),
        // so a group's count and number fit in 16 bits.  Targets are grouped
        // in an open-addressing table (target -> group, groups numbered by
        // first appearance) of at least twice that many entries.
        std::vector<Contribution> buf;
        int bits = 4;
        while ((int64_t(1) << bits) < 4 * (int64_t)CH * NL) ++bits;
        std::vector<int32_t> hkey(size_t(1) << bits, -1), hgroup(size_t(1) << bits);
        std::vector<uint32_t> gslot;
        std::vector<int32_t> group_of, gtarget, gmirror, gcount;
        std::vector<uint64_t> gorder;   // (65535 - count, target, group), ascending
        std::vector<size_t> gstart;
        for (int64_t pi = part_begin; pi < part_end; ++pi) {
            Part& out = parts[pi];
            const int64_t k0 = pi * per, k1 = std::min<int64_t>(p.n_chunks, k0 + per);
            for (int64_t k = k0; k < k1; ++k) {
                const int64_t i0 = k * CH, i1 = std::min<int64_t>(E, i0 + CH);
                buf.clear();
                for (int64_t i = i0; i < i1; ++i) {
                    const int el = (int)(i - i0);
                    const int64_t e = p.perm[i];
                    const int32_t* c = p.conn.data() + i * B;
                    if (matrix) {
                        int l = 0;
                        for (int a = 0; a < B; ++a)
                            for (int b = a; b < B; ++b, ++l) {
                                const int64_t pab = p.slot[(e * B + a) * B + b];
                                const int64_t pba = p.slot[(e * B + b) * B + a];
                                const uint16_t code = (uint16_t)((el * NL + l) << 1);
                                if (c[a] < c[b]) {
                                    buf.push_back({(int32_t)pab, (int32_t)pba, code});
                                } else if (c[a] > c[b]) {
                                    buf.push_back({(int32_t)pba, (int32_t)pab, (uint16_t)(code | 1)});
                                } else {
                                    buf.push_back({(int32_t)pab, (int32_t)pab, code});
                                    if (a != b) buf.push_back({(int32_t)pab, (int32_t)pab, (uint16_t)(code | 1)});
                                }
                            }
                    } else {
                        for (int a = 0; a < B; ++a) buf.push_back({c[a], -1, (uint16_t)((el * NL + a) << 1)});
                    }
                }
                // one group (slot) per target; targets are non-negative
                gslot.clear();
                gtarget.clear();
                gmirror.clear();
                gcount.clear();
                group_of.resize(buf.size());
                for (size_t q = 0; q < buf.size(); ++q) {
                    const int32_t t = buf[q].target;
                    uint32_t h = ((uint32_t)t * 2654435761u) >> (32 - bits);
                    while (hkey[h] != -1 && hkey[h] != t) h = (h + 1) & ((1u << bits) - 1);
                    if (hkey[h] == -1) {
                        hkey[h] = t;
                        hgroup[h] = (int32_t)gtarget.size();
                        gslot.push_back(h);
                        gtarget.push_back(t);
                        gmirror.push_back(buf[q].mirror);
                        gcount.push_back(0);
                    }
                    group_of[q] = hgroup[h];
                    ++gcount[hgroup[h]];
                }
                for (const uint32_t h : gslot) hkey[h] = -1;
                // slots by decreasing contribution count, so that the threads
                // of a warp (one slot each) loop equally long, then by target;
                // a slot's contributions keep their (element, entry) order
                const size_t G = gtarget.size();
                gorder.resize(G);
                for (size_t g = 0; g < G; ++g)
                    gorder[g] = (uint64_t)(65535 - gcount[g]) << 48 | (uint64_t)gtarget[g] << 16 | g;
                std::sort(gorder.begin(), gorder.end());
                const size_t s0 = out.slot_target.size(), c0 = out.contrib.size();
                out.slot_target.resize(s0 + G);
                out.slot_mirror.resize(s0 + G);
                out.slot_len.resize(s0 + G);
                out.contrib.resize(c0 + buf.size());
                gstart.resize(G);
                for (size_t i = 0, c = c0; i < G; ++i) {
                    const size_t g = gorder[i] & 0xFFFF;
                    out.slot_target[s0 + i] = gtarget[g];
                    out.slot_mirror[s0 + i] = gmirror[g];
                    out.slot_len[s0 + i] = gcount[g];
                    gstart[g] = c;
                    c += gcount[g];
                }
                for (size_t q = 0; q < buf.size(); ++q) out.contrib[gstart[group_of[q]]++] = buf[q].code;
                out.chunk_slots.push_back((int32_t)G);
            }
        }
    });
    // concatenate in chunk order
    std::vector<size_t> so(n_parts + 1, 0), co(n_parts + 1, 0);
    for (int q = 0; q < n_parts; ++q) {
        so[q + 1] = so[q] + parts[q].slot_target.size();
        co[q + 1] = co[q] + parts[q].contrib.size();
    }
    const size_t n_slots = so[n_parts], n_contrib = co[n_parts];
    if (n_slots > (size_t)INT32_MAX || n_contrib > (size_t)INT32_MAX) return TM_ERR_TOO_LARGE;
    p.chunk_begin.assign(p.n_chunks + 1, 0);
    p.slot_target.resize(n_slots);
    p.slot_mirror.resize(n_slots);
    p.slot_ptr.resize(n_slots + 1);
    p.slot_ptr[0] = 0;
    p.contrib.resize(n_contrib);
    parallel_for(n_parts, T, [&](int64_t q0, int64_t q1) {
        for (int64_t q = q0; q < q1; ++q) {
            const Part& pt = parts[q];
            std::copy(pt.slot_target.begin(), pt.slot_target.end(), p.slot_target.begin() + so[q]);
            std::copy(pt.slot_mirror.begin(), pt.slot_mirror.end(), p.slot_mirror.begin() + so[q]);
            std::copy(pt.contrib.begin(), pt.contrib.end(), p.contrib.begin() + co[q]);
            size_t c = co[q];
            for (size_t j = 0; j < pt.slot_len.size(); ++j) {
                c += pt.slot_len[j];
                p.slot_ptr[so[q] + j + 1] = (int32_t)c;
            }
        }
    });
    {
        int64_t k = 0;
        for (const Part& pt : parts)
            for (const int32_t ns : pt.chunk_slots) {
                p.chunk_begin[k + 1] = p.chunk_begin[k] + ns;
                ++k;
            }
    }
    parts.clear();
    // partials per target (the chunks that touch it) and, for the matrix,
    // the mirror of every target: counts commute, so relaxed atomic adds on
    // host threads give the same counts for any number of threads, and all
    // slots of one target carry the same mirror
    buffer<int32_t> chunks_per_target(n_targets);
    buffer<int32_t> mirror_of(matrix ? n_targets : 0);
    parallel_for(n_targets, T, [&](int64_t t0, int64_t t1) {
        std::fill(chunks_per_target.begin() + t0, chunks_per_target.begin() + t1, 0);
        if (matrix) std::fill(mirror_of.begin() + t0, mirror_of.begin() + t1, -1);
    }, kGrain);
    parallel_for((int64_t)n_slots, T, [&](int64_t s0, int64_t s1) {
        for (int64_t s = s0; s < s1; ++s) {
            const int32_t t = p.slot_target[s];
            __atomic_fetch_add(&chunks_per_target[t], 1, __ATOMIC_RELAXED);
            if (matrix) __atomic_store_n(&mirror_of[t], p.slot_mirror[s], __ATOMIC_RELAXED);
        }
    }, kGrain);
    // first contribution of every chunk, and the largest chunk, for kernels
    // that stage a chunk's slots and contributions in shared memory
    p.chunk_contrib.resize(p.chunk_begin.size());
    for (size_t k = 0; k < p.chunk_begin.size(); ++k) p.chunk_contrib[k] = p.slot_ptr[p.chunk_begin[k]];
    for (size_t k = 0; k + 1 < p.chunk_begin.size(); ++k) {
        p.max_chunk_slots = std::max(p.max_chunk_slots, p.chunk_begin[k + 1] - p.chunk_begin[k]);
        p.max_chunk_contrib = std::max(p.max_chunk_contrib, p.chunk_contrib[k + 1] - p.chunk_contrib[k]);
    }
    // shared targets (touched by more than one chunk), numbered by
    // decreasing partial count and then by target (neighbouring threads of
    // the finalizing kernel loop equally long); their partials are
    // contiguous per target and ordered by chunk.  The numbering is a stable
    // counting sort on the count over ranges of targets on host threads; the
    // histograms (ranges x counts) stay within n_targets entries.
    int32_t max_count = 0;
    for (int64_t t = 0; t < n_targets; ++t) max_count = std::max(max_count, chunks_per_target[t]);
    const int64_t W = (int64_t)max_count + 1;
    const int64_t R = std::max<int64_t>(1, std::min<int64_t>(T, n_targets / std::max<int64_t>(W, kGrain)));
    const int64_t tstep = std::max<int64_t>(1, (n_targets + R - 1) / R);
    std::vector<int64_t> hist((size_t)(R * W), 0);
    parallel_for(R, T, [&](int64_t r0, int64_t r1) {
        for (int64_t r = r0; r < r1; ++r)
            for (int64_t t = r * tstep; t < std::min(n_targets, (r + 1) * tstep); ++t)
                if (chunks_per_target[t] > 1) ++hist[r * W + chunks_per_target[t]];
    });
    // offsets in the order (count descending, range, target), and the first
    // index and first partial of every count
    std::vector<int64_t> class_first(W, 0), class_partial(W, 0);
    int64_t n_shared = 0, n_partials = 0;
    for (int64_t c = W - 1; c >= 2; --c) {
        class_first[c] = n_shared;
        class_partial[c] = n_partials;
        for (int64_t r = 0; r < R; ++r) {
            const int64_t h = hist[r * W + c];
            hist[r * W + c] = n_shared;
            n_shared += h;
        }
        n_partials += (n_shared - class_first[c]) * c;
    }
    buffer<int32_t> shared_index(n_targets);
    p.shared_target.resize(n_shared);
    p.shared_mirror.resize(n_shared);
    p.shared_ptr.resize(n_shared + 1);
    parallel_for(R, T, [&](int64_t r0, int64_t r1) {
        for (int64_t r = r0; r < r1; ++r)
            for (int64_t t = r * tstep; t < std::min(n_targets, (r + 1) * tstep); ++t) {
                const int32_t c = chunks_per_target[t];
                if (c > 1) {
                    const int64_t i = hist[r * W + c]++;
                    shared_index[t] = (int32_t)i;
                    p.shared_target[i] = (int32_t)t;
                    p.shared_mirror[i] = matrix ? mirror_of[t] : -1;
                    p.shared_ptr[i] = (int32_t)(class_partial[c] + (i - class_first[c]) * c);
                } else {
                    shared_index[t] = -1;
                }
            }
    });
    p.shared_ptr[n_shared] = (int32_t)n_partials;
    p.n_partials = n_partials;
    // a shared slot's partial is the next one of its target in slot (=
    // chunk) order.  Host threads own ranges of shared targets holding about
    // equal numbers of partials and each scans all slots, so the counter of
    // every target advances in slot order on one thread.
    buffer<int32_t> slot_shared(n_slots);
    parallel_for((int64_t)n_slots, T, [&](int64_t s0, int64_t s1) {
        for (int64_t s = s0; s < s1; ++s) slot_shared[s] = shared_index[p.slot_target[s]];
    }, kGrain);
    const int64_t TO = std::max<int64_t>(1, std::min<int64_t>({(int64_t)T, n_shared, (int64_t)n_slots / kGrain}));
    std::vector<int64_t> own(TO + 1, n_shared);
    for (int64_t o = 0; o < TO; ++o)
        own[o] = std::lower_bound(p.shared_ptr.begin(), p.shared_ptr.begin() + n_shared, n_partials * o / TO) -
                 p.shared_ptr.begin();
    buffer<int32_t> next(n_shared);
    parallel_for(TO, T, [&](int64_t o0, int64_t o1) {
        for (int64_t o = o0; o < o1; ++o) {
            const int32_t lo = (int32_t)own[o], n_own = (int32_t)(own[o + 1] - own[o]);
            if (n_own <= 0) continue;
            for (int32_t sh = lo; sh < lo + n_own; ++sh) next[sh] = p.shared_ptr[sh];
            for (size_t s = 0; s < n_slots; ++s) {
                const int32_t sh = slot_shared[s];
                if ((uint32_t)(sh - lo) < (uint32_t)n_own) {
                    p.slot_target[s] = -(next[sh]++ + 1);
                    p.slot_mirror[s] = sh;
                }
            }
        }
    });
    return TM_OK;
}

}  // namespace

namespace {

uint64_t spread_bits(uint64_t x, int dims) {
    if (dims == 2) {
        x &= 0xFFFFFFFFull;
        x = (x | (x << 16)) & 0x0000FFFF0000FFFFull;
        x = (x | (x << 8)) & 0x00FF00FF00FF00FFull;
        x = (x | (x << 4)) & 0x0F0F0F0F0F0F0F0Full;
        x = (x | (x << 2)) & 0x3333333333333333ull;
        x = (x | (x << 1)) & 0x5555555555555555ull;
        return x;
    }
    x &= 0x1FFFFFull;
    x = (x | (x << 32)) & 0x1F00000000FFFFull;
    x = (x | (x << 16)) & 0x1F0000FF0000FFull;
    x = (x | (x << 8)) & 0x100F00F00F00F00Full;
    x = (x | (x << 4)) & 0x10C30C30C30C30C3ull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}

}  // namespace

extern "C" int tm_morton_order(const double* points, int64_t n_points, int32_t dim, const int64_t* conn,
                               int64_t n_elements, int32_t n_basis, int32_t* perm) {
    if (n_elements < 0 || n_points < 0 || (dim != 2 && dim != 3) || n_basis < dim + 1 ||
        (n_elements > 0 && (!points || !conn || !perm)))
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_morton_order: bad arguments");
    if (n_elements > INT32_MAX) return tm_set_error(TM_ERR_TOO_LARGE, "tm_morton_order: more than 2^31 elements");
    if (n_elements == 0) return TM_OK;
    const int D = dim, V = dim + 1;
    for (int64_t k = 0; k < n_elements * n_basis; ++k)
        if (conn[k] < 0 || conn[k] >= n_points)
            return tm_set_error(TM_ERR_INVALID_ARG, "tm_morton_order: connectivity index out of range");
    try {
        const int T = host_threads();
        // centroid of the vertices ((x0 + x1) + x2 ...) / (D + 1), and their box
        std::vector<double> cent((size_t)n_elements * D);
        parallel_for(n_elements, T, [&](int64_t e0, int64_t e1) {
            for (int64_t e = e0; e < e1; ++e)
                for (int d = 0; d < D; ++d) {
                    double s = points[conn[e * n_basis] * D + d];
                    for (int v = 1; v < V; ++v) s += points[conn[e * n_basis + v] * D + d];
                    cent[e * D + d] = s / (double)V;
                }
        }, kGrain / 4);
        double lo[3], hi[3], span[3];
        for (int d = 0; d < D; ++d) {
            lo[d] = hi[d] = cent[d];
            for (int64_t e = 1; e < n_elements; ++e) {
                lo[d] = std::min(lo[d], cent[e * D + d]);
                hi[d] = std::max(hi[d], cent[e * D + d]);
            }
            span[d] = hi[d] > lo[d] ? hi[d] - lo[d] : 1.0;
        }
        const int bits = D == 2 ? 31 : 21;
        const double scale = (double)((1ll << bits) - 1);
        std::vector<std::pair<uint64_t, int32_t>> key((size_t)n_elements);
        parallel_for(n_elements, T, [&](int64_t e0, int64_t e1) {
            for (int64_t e = e0; e < e1; ++e) {
                uint64_t k = 0;
                for (int d = 0; d < D; ++d) {
                    const double q = std::floor((cent[e * D + d] - lo[d]) / span[d] * scale);
                    k |= spread_bits((uint64_t)q, D) << d;
                }
                key[e] = {k, (int32_t)e};
            }
        }, kGrain / 4);
        // sort ranges on host threads, then merge; (key, index) pairs give
        // the stable order
        const int TS = threads_for(n_elements, kGrain);
        const int64_t step = (n_elements + TS - 1) / TS;
        parallel_for(TS, TS, [&](int64_t t0, int64_t t1) {
            for (int64_t t = t0; t < t1; ++t) {
                const int64_t b = std::min(n_elements, t * step), e = std::min(n_elements, (t + 1) * step);
                std::sort(key.begin() + b, key.begin() + e);
            }
        });
        for (int64_t w = step; w < n_elements; w *= 2)
            for (int64_t b = 0; b + w < n_elements; b += 2 * w)
                std::inplace_merge(key.begin() + b, key.begin() + b + w,
                                   key.begin() + std::min(n_elements, b + 2 * w));
        for (int64_t e = 0; e < n_elements; ++e) perm[e] = key[e].second;
    } catch (const std::bad_alloc&) {
        return tm_set_error(TM_ERR_PLAN, "tm_morton_order: out of host memory");
    }
    return TM_OK;
}

extern "C" int tm_plan_build(const int64_t* conn, int64_t n_elements, int32_t n_basis,
                             int64_t n_points, int32_t kind, int32_t chunk_elems,
                             const int32_t* perm, const int64_t* slot_map, tm_host_plan** out) {
    if (!out) return tm_set_error(TM_ERR_INVALID_ARG, "tm_plan_build: out is null");
    *out = nullptr;
    if (n_elements < 0 || n_basis < 1 || n_basis > 10 || n_points < 0 || chunk_elems < 1 ||
        (kind != TM_PLAN_KIND_MATRIX && kind != TM_PLAN_KIND_NODE) || (n_elements > 0 && !conn))
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_plan_build: bad arguments");
    if (n_points > INT32_MAX || n_elements > INT32_MAX)
        return tm_set_error(TM_ERR_TOO_LARGE, "tm_plan_build: more than 2^31 nodes or elements");
    tm_host_plan* p = new (std::nothrow) tm_host_plan();
    if (!p) return tm_set_error(TM_ERR_PLAN, "tm_plan_build: out of host memory");
    try {
        p->kind = kind;
        p->n_elements = n_elements;
        p->n_basis = n_basis;
        p->n_points = n_points;
        p->chunk_elems = chunk_elems;
        p->n_local = kind == TM_PLAN_KIND_MATRIX ? n_basis * (n_basis + 1) / 2 : n_basis;
        const int T = host_threads();
        std::atomic<bool> bad_index(false);
        parallel_for(n_elements * n_basis, T, [&](int64_t k0, int64_t k1) {
            for (int64_t k = k0; k < k1; ++k)
                if (conn[k] < 0 || conn[k] >= n_points) {
                    bad_index = true;
                    return;
                }
        }, kGrain);
        if (bad_index) {
            delete p;
            return tm_set_error(TM_ERR_INVALID_ARG, "tm_plan_build: connectivity index out of range");
        }
        p->perm.resize(n_elements);
        if (perm) {
            std::vector<char> seen(n_elements, 0);
            for (int64_t i = 0; i < n_elements; ++i) {
                if (perm[i] < 0 || perm[i] >= n_elements || seen[perm[i]]) {
                    delete p;
                    return tm_set_error(TM_ERR_INVALID_ARG, "tm_plan_build: perm is not a permutation");
                }
                seen[perm[i]] = 1;
                p->perm[i] = perm[i];
            }
        } else {
            std::iota(p->perm.begin(), p->perm.end(), 0);
        }
        p->conn.resize((size_t)n_elements * n_basis);
        parallel_for(n_elements, T, [&](int64_t i0, int64_t i1) {
            for (int64_t i = i0; i < i1; ++i)
                for (int a = 0; a < n_basis; ++a)
                    p->conn[i * n_basis + a] = (int32_t)conn[(int64_t)p->perm[i] * n_basis + a];
        }, kGrain / 4);
        if (kind == TM_PLAN_KIND_MATRIX) {
            if (slot_map) {
                const int64_t n_slot = n_elements * n_basis * n_basis;
                p->slot.resize(n_slot);
                const int TS = threads_for(n_slot, kGrain);
                std::vector<int64_t> range_max(TS, -1), range_min(TS, 0);
                const int64_t step = (n_slot + TS - 1) / TS;
                parallel_for(TS, TS, [&](int64_t t0, int64_t t1) {
                    for (int64_t t = t0; t < t1; ++t) {
                        const int64_t b = std::min(n_slot, t * step), e = std::min(n_slot, b + step);
                        std::copy(slot_map + b, slot_map + e, p->slot.begin() + b);
                        // the range's extremes in registers, stored once (the
                        // per-thread entries share cache lines)
                        int64_t mx = -1, mn = 0;
                        for (int64_t k = b; k < e; ++k) {
                            mx = std::max(mx, slot_map[k]);
                            mn = std::min(mn, slot_map[k]);
                        }
                        range_max[t] = mx;
                        range_min[t] = mn;
                    }
                });
                if (*std::min_element(range_min.begin(), range_min.end()) < 0) {
                    delete p;
                    return tm_set_error(TM_ERR_INVALID_ARG, "tm_plan_build: negative slot_map entry");
                }
                p->nnz = *std::max_element(range_max.begin(), range_max.end()) + 1;
            } else {
                build_pattern(*p, conn);
            }
            if (p->nnz > INT32_MAX) {
                delete p;
                return tm_set_error(TM_ERR_TOO_LARGE, "tm_plan_build: more than 2^31 CSR entries");
            }
        }
        const int st = build_chunks(*p);
        if (st != TM_OK) {
            delete p;
            return tm_set_error(st, "tm_plan_build: chunk_elems * n_local * 2 exceeds 65536");
        }
    } catch (const std::bad_alloc&) {
        delete p;
        return tm_set_error(TM_ERR_PLAN, "tm_plan_build: out of host memory");
    }
    *out = p;
    return TM_OK;
}

extern "C" int64_t tm_plan_array_size(const tm_host_plan* p, int32_t id) {
    if (!p) return -1;
    switch (id) {
        case TM_PLAN_EDGE_ROW: return (int64_t)p->edge_row.size();
        case TM_PLAN_EDGE_COL: return (int64_t)p->edge_col.size();
        case TM_PLAN_SLOT: return (int64_t)p->slot.size();
        case TM_PLAN_CHUNK_BEGIN: return (int64_t)p->chunk_begin.size();
        case TM_PLAN_SLOT_PTR: return (int64_t)p->slot_ptr.size();
        case TM_PLAN_CONTRIB: return (int64_t)p->contrib.size();
        case TM_PLAN_SLOT_TARGET: return (int64_t)p->slot_target.size();
        case TM_PLAN_SLOT_MIRROR: return (int64_t)p->slot_mirror.size();
        case TM_PLAN_SHARED_PTR: return (int64_t)p->shared_ptr.size();
        case TM_PLAN_SHARED_TARGET: return (int64_t)p->shared_target.size();
        case TM_PLAN_SHARED_MIRROR: return (int64_t)p->shared_mirror.size();
        case TM_PLAN_CONN: return (int64_t)p->conn.size();
        case TM_PLAN_PERM: return (int64_t)p->perm.size();
        case TM_PLAN_CHUNK_CONTRIB: return (int64_t)p->chunk_contrib.size();
        default: return -1;
    }
}

// copies in 4 MB pieces on host threads: the caller's fresh destination
// pages are first touched in parallel
template <typename T>
static int copy_vec(const buffer<T>& v, void* dst) {
    const int64_t n = (int64_t)v.size() * (int64_t)sizeof(T), piece = 4 << 20;
    try {
        parallel_for((n + piece - 1) / piece, host_threads(), [&](int64_t q0, int64_t q1) {
            const int64_t b = q0 * piece, e = std::min(n, q1 * piece);
            std::memcpy((char*)dst + b, (const char*)v.data() + b, (size_t)(e - b));
        });
    } catch (...) {
        return tm_set_error(TM_ERR_PLAN, "tm_plan_copy_array: out of host memory");
    }
    return TM_OK;
}

extern "C" int tm_plan_copy_array(const tm_host_plan* p, int32_t id, void* dst) {
    if (!p || (!dst && tm_plan_array_size(p, id) > 0))
        return tm_set_error(TM_ERR_INVALID_ARG, "tm_plan_copy_array: null argument");
    switch (id) {
        case TM_PLAN_EDGE_ROW: return copy_vec(p->edge_row, dst);
        case TM_PLAN_EDGE_COL: return copy_vec(p->edge_col, dst);
        case TM_PLAN_SLOT: return copy_vec(p->slot, dst);
        case TM_PLAN_CHUNK_BEGIN: return copy_vec(p->chunk_begin, dst);
        case TM_PLAN_SLOT_PTR: return copy_vec(p->slot_ptr, dst);
        case TM_PLAN_CONTRIB: return copy_vec(p->contrib, dst);
        case TM_PLAN_SLOT_TARGET: return copy_vec(p->slot_target, dst);
        case TM_PLAN_SLOT_MIRROR: return copy_vec(p->slot_mirror, dst);
        case TM_PLAN_SHARED_PTR: return copy_vec(p->shared_ptr, dst);
        case TM_PLAN_SHARED_TARGET: return copy_vec(p->shared_target, dst);
        case TM_PLAN_SHARED_MIRROR: return copy_vec(p->shared_mirror, dst);
        case TM_PLAN_CONN: return copy_vec(p->conn, dst);
        case TM_PLAN_PERM: return copy_vec(p->perm, dst);
        case TM_PLAN_CHUNK_CONTRIB: return copy_vec(p->chunk_contrib, dst);
        default: return tm_set_error(TM_ERR_INVALID_ARG, "tm_plan_copy_array: unknown array id");
    }
}

extern "C" int64_t tm_plan_scalar(const tm_host_plan* p, int32_t which) {
    if (!p) return -1;
    switch (which) {
        case 0: return p->nnz;
        case 1: return p->n_chunks;
        case 2: return (int64_t)p->slot_target.size();
        case 3: return (int64_t)p->contrib.size();
        case 4: return (int64_t)p->shared_target.size();
        case 5: return p->n_partials;
        case 6: return p->n_local;
        case 7: return p->max_chunk_slots;
        case 8: return p->max_chunk_contrib;
        default: return -1;
    }
}

extern "C" void tm_plan_free(tm_host_plan* p) { delete p; }
