// pjg_kernels.cu — device kernels of libpjg (sm_103a).
//
// The search replaces Jess's per-pair Scanner (patches/Scanner.c.patch:
// 110-336) + KdTree range queries (patches/KdTree.c.patch:226-298) +
// superposition (patches/Super.c.patch) with:
//
//   k_params            annulus radii of every ordered template-atom pair
//   k_candidate_counts  candidate-list lengths per (structure, signature)
//                       from the per-bucket histograms of atom names
//   k_candidates        the lists themselves, in candidate (ResIndex) order
//   k_scan_*            exclusive scans of list lengths and row counts
//   k_axis_ranks        per-structure axis ranks (once, at upload)
//   k_demand_levels     requests the kd leaf order of the lists a pair
//                       reaches first
//   k_list_keys, k_list_reps, k_list_share
//                       requested lists with the same atoms share one
//                       leaf order
//   k_leaf_part<M>      kd leaf order of tie-free lists by axis partitions
//                       of presorted orders (tied or longer lists are
//                       passed on; k_leaf_order, the rank method, in the
//                       PJG_LEAF_RANK build)
//   k_leaf_sorted<M>    kd leaf order by sorted-axis splits, with a qselect
//                       replay of tied nodes
//   k_leaf_exact<M>     the literal qselect sequence, for the rest
//   k_search            persistent warp per pair, order-preserving
//                       depth-first-over-tiles frontier expansion
//                       (k_search_large: templates over 32 atoms)
//   k_superpose         thread per complete row, FP64 covariance and
//                       quaternion eigen-solve
//   k_order_counts, k_automaton, k_gather_hits
//                       Query.__next__ per pair and compaction of the hits
//
// FP64 arithmetic that decides a hit is written with __dadd_rn/__dsub_rn/
// __dmul_rn so it is never contracted into FMA and matches the reference's
// (x86-64, unfused) operation order bit for bit.

#include <cuda_runtime.h>

#include <cfloat>
#include <climits>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <algorithm>

#include "pjg_common.cuh"
#include "pjg_kernels.cuh"

namespace pjg {

#define FULL_MASK 0xffffffffu

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// ---------------------------------------------------------------------------
// k_params: AnnulusParam for every ordered pair (p, q) of every template.
// Scanner_next (patches/Scanner.c.patch:308-325): theta = (r + w_p) + w_q
// clipped to s, min = d - theta, max = d + theta, min raised to 0.5;
// Annulus_reuse (patches/Annulus.c.patch:107-139): swap if b < a, clamp at
// 0, squares a*a and b*b, box half-width b.

__global__ void k_params(int n_templates, const int32_t *atom_begin, const int32_t *param_begin,
                         const double *dist, const double *weight, double r, double s, double g,
                         AnnulusParam *out) {
    int t = blockIdx.x;
    if (t >= n_templates) return;
    int a0 = atom_begin[t];
    int n = atom_begin[t + 1] - a0;
    int base = param_begin[t];
    for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
        int p = idx / n, q = idx % n;
        double d = dist[base + idx];
        double theta = __dadd_rn(__dadd_rn(r, weight[a0 + p]), weight[a0 + q]);
        if (theta > s) theta = s;
        double mn = __dsub_rn(d, theta);
        double mx = __dadd_rn(d, theta);
        if (mn < 0.5) mn = 0.5;
        double a = mn, b = mx;
        if (b < a) {
            double tmp = a;
            a = b;
            b = tmp;
        }
        if (a < 0.0) a = 0.0;
        if (b < 0.0) b = 0.0;
        AnnulusParam P;
        P.a2 = __dmul_rn(a, a);
        P.b2 = __dmul_rn(b, b);
        P.b = b;
        double alo = a - g, ahi = a + g, blo = b - g, bhi = b + g;
        P.thr.x = alo > 0.0 ? __double2float_rd(alo * alo) : -1.0f;
        P.thr.y = __double2float_ru(ahi * ahi);
        P.thr.z = blo > 0.0 ? __double2float_rd(blo * blo) : -1.0f;
        P.thr.w = __double2float_ru(bhi * bhi);
        P.pad = 0.0;
        out[base + idx] = P;
    }
}

// ---------------------------------------------------------------------------
// Candidate rules.  TessTemplate_candidates (patches/TessTemplate.c.patch:
// 173-233): codes -1..8 walk the residue buckets of the template atom's
// residue names (first occurrence of each name only), in ResIndex order
// (residue name, then serial); other codes scan the molecule in order.

__device__ __forceinline__ bool in_list(uint32_t v, const uint32_t *list, int lo, int hi) {
    for (int i = lo; i < hi; i++)
        if (list[i] == v) return true;
    return false;
}

// "_CA_", "_N__", "_O__" as little-endian u32
__device__ __forceinline__ bool is_mainchain(uint32_t nm) {
    return nm == 0x5F41435Fu || nm == 0x5F5F4E5Fu || nm == 0x5F5F4F5Fu;
}

__device__ __forceinline__ bool sig_match(const SigView &sv, int g, int rule, uint32_t name,
                                          uint32_t resname) {
    int n0 = sv.name_begin[g], n1 = sv.name_begin[g + 1];
    switch (rule) {
    case RULE_ANY:
        return true;
    case RULE_NAME:
        return in_list(name, sv.names, n0, n1);
    case RULE_NAME_OR_PARTNER: {
        if (in_list(name, sv.names, n0, n1)) return true;
        for (int i = sv.partner_begin[g]; i < sv.partner_begin[g + 1]; i++)
            if (sv.partner_res[i] == resname && sv.partner_name[i] == name) return true;
        return false;
    }
    case RULE_NAME_OR_MAINCHAIN:
        if (in_list(name, sv.names, n0, n1)) return true;
        return sv.mainchain[g] && is_mainchain(name);
    case RULE_ELEMENT:
        for (int i = n0; i < n1; i++)
            if ((sv.names[i] & 0xFFFFu) == (name & 0xFFFFu)) return true;
        return false;
    }
    return false;
}

// A signature's rule with up to four of its names held in registers (read
// once per list instead of once per scanned atom).
struct SigRegs {
    int g, rule, n0, n1, mainchain;
    uint32_t nm[4];
};

__device__ __forceinline__ SigRegs load_sig(const SigView &sv, int g) {
    SigRegs r;
    r.g = g;
    r.rule = sv.rule[g];
    r.n0 = sv.name_begin[g];
    r.n1 = sv.name_begin[g + 1];
    r.mainchain = sv.mainchain[g];
    for (int i = 0; i < 4; i++) r.nm[i] = r.n0 + i < r.n1 ? sv.names[r.n0 + i] : 0u;
    return r;
}

__device__ __forceinline__ bool sig_match_regs(const SigView &sv, const SigRegs &r, uint32_t name,
                                               uint32_t resname) {
    const int nn = r.n1 - r.n0;
    if (nn > 4) return sig_match(sv, r.g, r.rule, name, resname);
    switch (r.rule) {
    case RULE_ANY:
        return true;
    case RULE_NAME:
    case RULE_NAME_OR_PARTNER:
    case RULE_NAME_OR_MAINCHAIN: {
        bool hit = false;
#pragma unroll
        for (int i = 0; i < 4; i++) hit |= i < nn && r.nm[i] == name;
        if (hit) return true;
        if (r.rule == RULE_NAME_OR_MAINCHAIN) return r.mainchain && is_mainchain(name);
        if (r.rule == RULE_NAME_OR_PARTNER) {
            for (int i = sv.partner_begin[r.g]; i < sv.partner_begin[r.g + 1]; i++)
                if (sv.partner_res[i] == resname && sv.partner_name[i] == name) return true;
        }
        return false;
    }
    case RULE_ELEMENT: {
        bool hit = false;
#pragma unroll
        for (int i = 0; i < 4; i++) hit |= i < nn && (r.nm[i] & 0xFFFFu) == (name & 0xFFFFu);
        return hit;
    }
    }
    return false;
}

// One warp per (structure, signature): the list's atoms in candidate order
// at offset[w] (its length comes from k_candidate_counts).
// Lists filled: every list of the chunk (work == nullptr), or the n_work
// lists of `work`; with `claim`, a list is filled only by the warp that
// moves its fill state from 0 to 1 (lists already filled are skipped).
__global__ void k_candidates(ChunkView cv, SigView sv, const int64_t *offset, int32_t *cand_atom,
                             const int64_t *work, const unsigned long long *n_work, int32_t *fill_state,
                             int32_t claim) {
    int lane = lane_id();
    int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    int64_t total = work ? (int64_t)*n_work : (int64_t)cv.n_structures * sv.n_sigs;
    for (int64_t item = warp; item < total; item += nwarps) {
        const int64_t w = work ? work[item] : item;
        if (claim) {
            int taken = 0;
            if (lane == 0) taken = atomicCAS(&fill_state[w], 0, 1) != 0;
            if (__shfl_sync(FULL_MASK, taken, 0)) continue;
        }
        int s = (int)(w / sv.n_sigs);
        int g = (int)(w % sv.n_sigs);
        int code = sv.code[g];
        const SigRegs sr = load_sig(sv, g);
        int64_t abase = cv.atom_base[s];
        int nat = cv.atom_count[s];
        int cnt = 0;
        const int64_t out0 = offset[w];
        // atoms p_lo..p_hi of the residue bucket `rn` (via_sorted) or of
        // the molecule in order
        auto visit = [&](int p_lo, int p_hi, bool via_sorted, uint32_t rn) {
            for (int p0 = p_lo; p0 < p_hi; p0 += 32) {
                int p = p0 + lane;
                bool valid = p < p_hi;
                bool ok = false;
                int atom = 0;
                if (valid) {
                    atom = via_sorted ? cv.sorted[abase + p] : p;
                    const uint32_t res = via_sorted ? rn : cv.resname[abase + atom];
                    ok = sig_match_regs(sv, sr, cv.name[abase + atom], res);
                }
                unsigned m = __ballot_sync(FULL_MASK, ok);
                if (ok) cand_atom[out0 + cnt + __popc(m & ((1u << lane) - 1u))] = atom;
                cnt += __popc(m);
            }
        };
        if (code >= -1 && code <= 8) {
            int b0 = cv.bucket_begin[s], b1 = cv.bucket_begin[s + 1];
            for (int ri = sv.res_begin[g]; ri < sv.res_begin[g + 1]; ri++) {
                uint32_t rn = sv.resnames[ri];
                int found = -1;
                for (int bb = b0; bb < b1; bb += 32) {
                    int b = bb + lane;
                    unsigned m = __ballot_sync(FULL_MASK, b < b1 && cv.bucket_name[b] == rn);
                    if (m) {
                        found = bb + __ffs(m) - 1;
                        break;
                    }
                }
                if (found < 0) continue;
                // the rule over the bucket's distinct atom names, as a bit
                // mask indexed by each atom's name index: a bit test per
                // atom, and no scan at all of a bucket with no passing name
                const int nb = cv.nh_begin[found], nd = cv.nh_begin[found + 1] - nb;
                if (nd > 64) {
                    visit(cv.bucket_lo[found], cv.bucket_hi[found], true, rn);
                    continue;
                }
                const bool m0 = lane < nd && sig_match_regs(sv, sr, cv.nh_name[nb + lane], rn);
                const bool m1 = lane + 32 < nd && sig_match_regs(sv, sr, cv.nh_name[nb + 32 + lane], rn);
                const uint64_t mask =
                    (uint64_t)__ballot_sync(FULL_MASK, m0) | ((uint64_t)__ballot_sync(FULL_MASK, m1) << 32);
                const int p_lo = cv.bucket_lo[found], p_hi = cv.bucket_hi[found];
                if (!mask) continue;
                if (__popcll((long long)mask) == 1) {
                    // one passing name: its atoms, already grouped in
                    // ResIndex order, copied as they are
                    const int q = nb + __ffsll((long long)mask) - 1;
                    const int cq = cv.nh_count[q];
                    const int32_t *src = cv.nh_pos + abase + cv.nh_off[q];
                    for (int i = lane; i < cq; i += 32) cand_atom[out0 + cnt + i] = src[i];
                    cnt += cq;
                    continue;
                }
                for (int p0 = p_lo; p0 < p_hi; p0 += 32) {
                    const int p = p0 + lane;
                    int atom = 0;
                    bool ok = false;
                    if (p < p_hi) {
                        atom = cv.sorted[abase + p];
                        ok = (mask >> cv.name_id[abase + atom]) & 1ull;
                    }
                    const unsigned m = __ballot_sync(FULL_MASK, ok);
                    if (ok) cand_atom[out0 + cnt + __popc(m & ((1u << lane) - 1u))] = atom;
                    cnt += __popc(m);
                }
            }
        } else {
            visit(0, nat, false, 0u);
        }
    }
}


// List lengths without scanning atoms.  Whether an atom joins a list
// depends only on its (residue name, atom name) and the signature, so a
// list's length is the sum, over the distinct atom names of each residue
// bucket it walks, of the counts of the names that pass the rule (the
// molecule-order codes walk every bucket of the structure).  Thread per
// (structure, signature): consecutive threads take consecutive signatures of
// one structure, so the structure's bucket tables are read by the whole warp
// at once.
__global__ void k_candidate_counts(ChunkView cv, SigView sv, int32_t *count, int32_t *scanned) {
    const int64_t total = (int64_t)cv.n_structures * sv.n_sigs;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < total; w += stride) {
        const int s = (int)(w / sv.n_sigs);
        const int g = (int)(w % sv.n_sigs);
        const int code = sv.code[g];
        const SigRegs sr = load_sig(sv, g);
        const int b0 = cv.bucket_begin[s], b1 = cv.bucket_begin[s + 1];
        int cnt = 0, sc = 0;
        auto bucket_sum = [&](int b, uint32_t rn) {
            const int q1 = cv.nh_begin[b + 1];
            for (int q = cv.nh_begin[b]; q < q1; q++)
                if (sig_match_regs(sv, sr, cv.nh_name[q], rn)) cnt += cv.nh_count[q];
        };
        if (code >= -1 && code <= 8) {
            for (int ri = sv.res_begin[g]; ri < sv.res_begin[g + 1]; ri++) {
                const uint32_t rn = sv.resnames[ri];
                int b = b0;
                while (b < b1 && cv.bucket_name[b] != rn) b++;
                if (b == b1) continue;
                bucket_sum(b, rn);
                sc += cv.bucket_hi[b] - cv.bucket_lo[b];
            }
        } else {
            for (int b = b0; b < b1; b++) bucket_sum(b, cv.bucket_name[b]);
            sc = cv.atom_count[s];
        }
        count[w] = cnt;
        scanned[w] = sc;
    }
}

// ---------------------------------------------------------------------------
// Exclusive scan (int32 -> int64), three phases.

constexpr int SCAN_THREADS = SCAN_TILE_THREADS;
constexpr int SCAN_ITEMS = SCAN_TILE_ITEMS / SCAN_TILE_THREADS;
constexpr int SCAN_TILE = SCAN_TILE_ITEMS;

__device__ int64_t block_exclusive_scan(int64_t v, int64_t *total) {
    __shared__ int64_t warp_sums[SCAN_THREADS / 32];
    int lane = lane_id(), wid = threadIdx.x >> 5;
    int64_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        int64_t y = __shfl_up_sync(FULL_MASK, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int64_t ws = lane < SCAN_THREADS / 32 ? warp_sums[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            int64_t y = __shfl_up_sync(FULL_MASK, ws, o);
            if (lane >= o) ws += y;
        }
        if (lane < SCAN_THREADS / 32) warp_sums[lane] = ws;
    }
    __syncthreads();
    int64_t before = wid ? warp_sums[wid - 1] : 0;
    *total = warp_sums[SCAN_THREADS / 32 - 1];
    __syncthreads();
    return before + x - v;
}

template <typename T>
__global__ void k_scan_tiles(const T *in, int64_t n, int64_t *out, int64_t *tile_sums) {
    int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
    int64_t v[SCAN_ITEMS];
    int64_t local = 0;
    for (int i = 0; i < SCAN_ITEMS; i++) {
        v[i] = base + i < n ? (int64_t)in[base + i] : 0;
        local += v[i];
    }
    int64_t total;
    int64_t ex = block_exclusive_scan(local, &total);
    for (int i = 0; i < SCAN_ITEMS; i++) {
        if (base + i < n) out[base + i] = ex;
        ex += v[i];
    }
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}


__global__ void k_scan_add(int64_t *out, int64_t n, const int64_t *tile_offsets) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += tile_offsets[i / SCAN_TILE];
}

// ---------------------------------------------------------------------------
// k_leaf_order: the order in which KdTreeQuery_next reports accepted leaves.
//
// KdTree_reuse / KdTreeNode_create (patches/KdTree.c.patch:157-205,
// 348-456) split a node of n points at n/2 with qselect_r on the axis
// x, y, z cycling, left child = first n/2 entries of the partitioned index
// array.  qselect_r (patches/qselect.h.patch:52-119) is median-of-3 pivot +
// Lomuto partition ("<= pivot" to the left), repeated until the pivot
// lands on k.  The query pushes the left child, then the right one, so the
// right subtree is popped first (pinned by the golden fixture): the DFS
// leaf order is the partitioned index array read backwards.  Pruning only
// removes subtrees, so accepted leaves always come out in this order.
//
// Fast paths (warp per list, shared memory): when no node has a tie at its
// median boundary (equal axis values on both sides of position n/2), each
// node's left/right sets are the n/2 smallest / the rest whatever the
// arrangement qselect leaves behind, so the leaf order follows from any
// recursive median split computed by all lanes.  Short lists use ranks
// (O(m^2) a level); longer ones sort each axis once and partition the three
// sorted arrays stably at every level (O(m) a level).  The FP32
// centroid-relative keys are a monotone rounding of the FP64 coordinates, so
// a tie there only sends the list to the exact path.  Exact path: the
// literal qselect replay on the FP64 coordinates (k_leaf_exact).  Each list
// also gets the bounding boxes of its blocks of CULL_BLK consecutive leaves (the
// search culls whole blocks against a parent's join box).

__device__ __forceinline__ int axis_cmp(double c, double d) { return c < d ? -1 : c > d ? 1 : 0; }

struct KdSel {
    const int32_t *atom;   // candidate-order atoms of the list
    const double *xyz;     // structure FP64 coordinates
    int axis;
    __device__ double key(int pos) const { return xyz[3 * (int64_t)atom[pos] + axis]; }
};

__device__ int qs_partition(int32_t *base, int left, int right, int pivot, const KdSel &S) {
    int store = left;
    int32_t t = base[right];
    base[right] = base[pivot];
    base[pivot] = t;
    double pv = S.key(base[right]);
    for (int i = left; i < right; i++) {
        if (axis_cmp(S.key(base[i]), pv) <= 0) {
            int32_t u = base[i];
            base[i] = base[store];
            base[store] = u;
            store++;
        }
    }
    t = base[store];
    base[store] = base[right];
    base[right] = t;
    return store;
}

__device__ int qs_median3(const int32_t *base, int left, int right, const KdSel &S) {
    int mid = (left + right + 1) / 2;
    double l = S.key(base[left]), r = S.key(base[right]), m = S.key(base[mid]);
    if ((axis_cmp(l, m) > 0) != (axis_cmp(l, r) > 0)) return left;
    if ((axis_cmp(m, l) < 0) != (axis_cmp(m, r) < 0)) return mid;
    return right;
}

__device__ void qselect(int32_t *base, int n, int k, const KdSel &S) {
    int left = 0, right = n - 1;
    for (;;) {
        if (left == right) return;
        int p = qs_median3(base, left, right, S);
        p = qs_partition(base, left, right, p, S);
        if (p == k) return;
        if (k < p) right = p - 1;
        else left = p + 1;
    }
}

// exact replay: perm[0..m) receives the partitioned candidate positions
__device__ __noinline__ void kd_exact(int32_t *perm, int m, const int32_t *ca, const double *xyz) {
    for (int i = 0; i < m; i++) perm[i] = i;
    KdSel S{ca, xyz, 0};
    int st_lo[40], st_n[40], st_ax[40];
    int sp = 1;
    st_lo[0] = 0;
    st_n[0] = m;
    st_ax[0] = 0;
    while (sp > 0) {
        sp--;
        int lo = st_lo[sp], n = st_n[sp], ax = st_ax[sp];
        if (n <= 1) continue;
        S.axis = ax;
        int split = n / 2;
        qselect(perm + lo, n, split, S);
        int nx = (ax + 1) % 3;
        st_lo[sp] = lo + split;
        st_n[sp] = n - split;
        st_ax[sp] = nx;
        sp++;
        st_lo[sp] = lo;
        st_n[sp] = split;
        st_ax[sp] = nx;
        sp++;
    }
}

template <int CAP>
struct LeafWarp {
    uint32_t ur[3][CAP];   // unique axis ranks by candidate index
    uint16_t lr[3][CAP];   // strict-lower axis ranks (low 16 bits: equal
                                     // ranks stay equal, a rare false tie only
                                     // sends the list to k_leaf_sorted)
    uint32_t cur[CAP];     // current axis unique rank in position order
    uint16_t ord[2][CAP];  // candidate index at each position
    uint16_t seg_lo[CAP];  // node (segment) of each position
    uint16_t seg_n[CAP];
    // level 0 by a bitmap over the structure's unique x ranks (a window of
    // 32 * LEAF_SORT_WORDS ranks at a time)
    uint32_t bits[LEAF_SORT_WORDS];
    uint16_t wpre[LEAF_SORT_WORDS];  // elements placed before each word
};

// Bounding boxes of the blocks of CULL_BLK consecutive leaves of a list
// (one warp; each 32-leaf step reduces CULL_BLK-lane segments).
__device__ void write_boxes(int m, int64_t o, const float4 *leaf_xyz, int64_t bo, float4 *blk_lo, float4 *blk_hi) {
    const int lane = lane_id();
    for (int b = 0; b * 32 < m; b++) {
        const int r = b * 32 + lane;
        const int first = r & ~(CULL_BLK - 1);  // first leaf of this lane's block
        float4 p = leaf_xyz[o + (r < m ? r : first < m ? first : b * 32)];
        float mnx = p.x, mny = p.y, mnz = p.z, mxx = p.x, mxy = p.y, mxz = p.z;
        for (int off = CULL_BLK / 2; off; off >>= 1) {
            mnx = fminf(mnx, __shfl_xor_sync(FULL_MASK, mnx, off));
            mny = fminf(mny, __shfl_xor_sync(FULL_MASK, mny, off));
            mnz = fminf(mnz, __shfl_xor_sync(FULL_MASK, mnz, off));
            mxx = fmaxf(mxx, __shfl_xor_sync(FULL_MASK, mxx, off));
            mxy = fmaxf(mxy, __shfl_xor_sync(FULL_MASK, mxy, off));
            mxz = fmaxf(mxz, __shfl_xor_sync(FULL_MASK, mxz, off));
        }
        if ((lane & (CULL_BLK - 1)) == 0 && first < m) {
            blk_lo[bo + r / CULL_BLK] = make_float4(mnx, mny, mnz, 0.f);
            blk_hi[bo + r / CULL_BLK] = make_float4(mxx, mxy, mxz, 0.f);
        }
    }
    __syncwarp();
}

__device__ void write_leaves(const uint16_t *order, int m, int64_t lo, const int32_t *ca, const float4 *pts,
                             int32_t *leaf_atom, float4 *leaf_xyz, int64_t bo, float4 *blk_lo, float4 *blk_hi) {
    const int lane = lane_id();
    for (int r = lane; r < m; r += 32) {
        int e = order[m - 1 - r];
        leaf_atom[lo + r] = ca[e];
        leaf_xyz[lo + r] = pts[ca[e]];
    }
    __syncwarp();
    write_boxes(m, lo, leaf_xyz, bo, blk_lo, blk_hi);
}

// The elements A[lo .. lo + n) in the order of their unique ranks on axis
// `ax`, into B[lo .. lo + n): a bitmap over the structure's ranks (windows of
// 32 * LEAF_SORT_WORDS), each element's place the set bits before it.
// False when an element was not placed once (a repeated atom).
template <int CAP>
__device__ bool sort_segment(LeafWarp<CAP> &L, const uint16_t *A, uint16_t *B, int lo, int n, int ax, int natoms) {
    const int lane = lane_id();
    constexpr int WB = 32 * LEAF_SORT_WORDS;
    int placed = 0;
    for (int wb = 0; wb < natoms; wb += WB) {
        const int nwords = min(LEAF_SORT_WORDS, (natoms - wb + 31) >> 5);
        for (int q = lane; q < nwords; q += 32) L.bits[q] = 0u;
        __syncwarp();
        for (int p = lo + lane; p < lo + n; p += 32) {
            const uint32_t u = L.ur[ax][A[p]] - (uint32_t)wb;
            if (u < (uint32_t)WB) atomicOr(&L.bits[u >> 5], 1u << (u & 31));
        }
        __syncwarp();
        int carry = placed;
        for (int w0 = 0; w0 < nwords; w0 += 32) {
            const int wd = w0 + lane;
            const int c = wd < nwords ? __popc(L.bits[wd]) : 0;
            int incl = c;
            for (int off = 1; off < 32; off <<= 1) {
                const int y = __shfl_up_sync(FULL_MASK, incl, off);
                if (lane >= off) incl += y;
            }
            if (wd < nwords) L.wpre[wd] = (uint16_t)(carry + incl - c);
            carry += __shfl_sync(FULL_MASK, incl, 31);
        }
        __syncwarp();
        for (int p = lo + lane; p < lo + n; p += 32) {
            const uint32_t u = L.ur[ax][A[p]] - (uint32_t)wb;
            if (u < (uint32_t)WB) {
                const uint32_t word = L.bits[u >> 5];
                const int pos = L.wpre[u >> 5] + __popc(word & ((1u << (u & 31)) - 1u));
                if (pos < n) B[lo + pos] = A[p];
            }
        }
        __syncwarp();
        placed = carry;
    }
    return placed == n;
}

// Leaf-order profile probes (PJG_SEARCH_PROF builds): every lane keeps the
// same per-warp sums (the probes sit on warp-uniform paths); lane 0 adds them
// to g_leaf_prof when the warp exits.
#if PJG_SEARCH_PROF
__device__ unsigned long long g_leaf_prof[LP_NUM];
#define LPROF_T(name) const long long name = clock64()
#define LPROF_ADD(i, v) (lp[i] += (unsigned long long)(v))
#else
#define LPROF_T(name)
#define LPROF_ADD(i, v) \
    do {                \
    } while (0)
#endif

__device__ __forceinline__ int leaf_class(int m) {
    return m <= 16 ? 0 : m <= 32 ? 1 : m <= 64 ? 2 : m <= 96 ? 3 : m <= 128 ? 4 : m <= 192 ? 5 : 6;
}

// Lists (at most rank_max <= CAP entries) without a tie: rank method, one
// warp per list -- the first levels by bitmap sorts of the nodes, the rest by
// counting each entry's smaller keys in its node.  Longer lists up to
// mid_max go to `mid_list` (the instance with larger buffers), longer or
// tied ones to k_leaf_sorted's worklists (up to LEAF_SORTED_MAX entries),
// the rest to k_leaf_exact's.  count_lists: this instance counts the lists it
// takes (the first one; the second sees lists the first already counted).
template <int CAP, int WARPS>
__global__ void __launch_bounds__(WARPS * 32)
    k_leaf_order(ChunkView cv, int32_t n_sigs, const int32_t *count, const int64_t *offset,
                 const int64_t *blk_offset, const int32_t *cand_atom, const int64_t *leaf_offset,
                 int32_t *leaf_atom, float4 *leaf_xyz, float4 *blk_lo, float4 *blk_hi, int64_t *sorted_list,
                 unsigned long long *sorted_count, int64_t list_cap, int64_t *exact_list,
                 unsigned long long *exact_count, unsigned long long *counters, int rank_max,
                 const int64_t *work, const unsigned long long *n_work, int64_t *mid_list,
                 unsigned long long *mid_count, int mid_max, int count_lists) {
    __shared__ LeafWarp<CAP> sh[WARPS];
    const int lane = lane_id();
    LeafWarp<CAP> &L = sh[threadIdx.x >> 5];
    int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    // the requested lists, or every list of the chunk
    int64_t total = work ? (int64_t)*n_work : (int64_t)cv.n_structures * n_sigs;
    unsigned long long n_exact = 0, n_sorted = 0, n_lists = 0, n_entries = 0;
#if PJG_SEARCH_PROF
    unsigned long long lp[LP_NUM] = {};
#endif
    for (int64_t item = warp; item < total; item += nwarps) {
        const int64_t w = work ? work[item] : item;
        const int m = count[w];
        if (m <= 0) continue;
        if (count_lists) {
            n_lists++;
            n_entries += (unsigned long long)m;
        }
        const int64_t o = offset[w];
        bool tie = m > rank_max;
        if (tie && mid_list && m <= mid_max) {
            if (lane == 0) mid_list[atomicAdd(mid_count, 1ull)] = w;
            __syncwarp();
            LPROF_ADD(LP_HANDED, 1);
            continue;
        }
        LPROF_T(t_list);
        int src = 0;
        if (!tie) {
            // keys: the atoms' unique axis ranks (an exact order of the FP64
            // coordinates, equal ones by atom index); a tie at a median
            // boundary is read from the strict-lower ranks
            const int64_t gbase = cv.atom_base[w / n_sigs];
            const int32_t *ca = cand_atom + o;
            for (int i = lane; i < m; i += 32) {
                const int64_t g = gbase + ca[i];
                for (int a = 0; a < 3; a++) {
                    L.ur[a][i] = cv.urank[a * cv.n_atoms + g];
                    L.lr[a][i] = (uint16_t)cv.lrank[a * cv.n_atoms + g];
                }
                L.ord[0][i] = (uint16_t)i;
                L.seg_lo[i] = 0;
                L.seg_n[i] = (uint16_t)m;
            }
            __syncwarp();
            for (int i = lane; i < m; i += 32) L.cur[i] = L.ur[0][i];
            __syncwarp();
            LPROF_T(t_load);
            LPROF_ADD(LP_CYC_LOAD, t_load - t_list);
            int levels = 0;
            while ((1 << levels) < m) levels++;
            for (int d = 0; d < levels; d++) {
                const uint16_t *A = L.ord[src];
                uint16_t *B = L.ord[src ^ 1];
                // the first levels of a longer list: each node in axis
                // order is the structure's axis order restricted to the node,
                // read from a bitmap over the unique axis ranks (what the
                // counting below computes, in O(atoms / 32 + m / 32) a node
                // instead of O(m n / 32))
                bool sorted0 = false;
                LPROF_T(t_a);
                if ((m >> d) >= LEAF_SORT_FROM) {
                    const int natoms = cv.atom_count[w / n_sigs];
                    sorted0 = true;
                    for (int lo = 0; lo < m;) {
                        const int n = L.seg_n[lo];
                        if (n <= 1) {
                            if (lane == 0) B[lo] = A[lo];
                        } else {
                            sorted0 = sort_segment(L, A, B, lo, n, d % 3, natoms) && sorted0;
                            LPROF_ADD(LP_SORT_NODES, 1);
                            LPROF_ADD(LP_SORT_WORDS, (natoms + 31) >> 5);
                        }
                        lo += n < 1 ? 1 : n;
                    }
                    __syncwarp();
                }
                LPROF_T(t_b);
                LPROF_ADD(LP_CYC_SORT, t_b - t_a);
                if (!sorted0) {
                    for (int p = lane; p < m; p += 32) {
                        const int lo = L.seg_lo[p], n = L.seg_n[p];
                        const int e = A[p];
                        if (n <= 1) {
                            B[p] = (uint16_t)e;
                            continue;
                        }
                        const uint32_t x = L.cur[p];
                        int before = 0;
#pragma unroll 8
                        for (int q = lo; q < lo + n; q++) before += L.cur[q] < x;
                        B[lo + before] = (uint16_t)e;
                        LPROF_ADD(LP_COUNT_PAIRS, n);
                    }
                }
                __syncwarp();
                LPROF_T(t_c);
                LPROF_ADD(LP_CYC_COUNT, t_c - t_b);
                // median-boundary ties, next axis keys, child nodes
                const int ax = d % 3, nax = (d + 1) % 3;
                bool t = false;
                for (int p = lane; p < m; p += 32) {
                    const int lo = L.seg_lo[p], n = L.seg_n[p];
                    const int e = B[p];
                    L.cur[p] = L.ur[nax][e];
                    if (n <= 1) continue;
                    const int k = n / 2;
                    if (p == lo + k && L.lr[ax][B[p - 1]] == L.lr[ax][e]) t = true;
                    if (p < lo + k) {
                        L.seg_n[p] = (uint16_t)k;
                    } else {
                        L.seg_lo[p] = (uint16_t)(lo + k);
                        L.seg_n[p] = (uint16_t)(n - k);
                    }
                }
                src ^= 1;
                __syncwarp();
                LPROF_T(t_d);
                LPROF_ADD(LP_CYC_SEG, t_d - t_c);
                if (__any_sync(FULL_MASK, t)) {
                    tie = true;
                    break;
                }
            }
        }
        if (tie) {
            LPROF_T(t_tie);
            LPROF_ADD(LP_CYC_LIST, t_tie - t_list);
            LPROF_ADD(LP_HANDED, 1);
            if (m <= LEAF_SORTED_MAX) {
                // size classes of k_leaf_sorted: up to 512, 1024, 2048 entries
                const int c = m <= 512 ? 0 : m <= 1024 ? 1 : 2;
                n_sorted++;
                if (lane == 0) sorted_list[c * list_cap + (int64_t)atomicAdd(&sorted_count[c], 1ull)] = w;
            } else {
                n_exact++;
                if (lane == 0) exact_list[atomicAdd(exact_count, 1ull)] = w;
            }
            __syncwarp();
            continue;
        }
        LPROF_T(t_w0);
        write_leaves(L.ord[src], m, leaf_offset[w], cand_atom + o, cv.xyz32 + cv.atom_base[w / n_sigs], leaf_atom,
                     leaf_xyz, blk_offset[w], blk_lo, blk_hi);
#if PJG_SEARCH_PROF
        {
            LPROF_T(t_w1);
            const int c = leaf_class(m);
            LPROF_ADD(LP_CYC_WRITE, t_w1 - t_w0);
            LPROF_ADD(LP_CYC_LIST, t_w1 - t_list);
            LPROF_ADD(LP_LISTS, 1);
            LPROF_ADD(LP_ENTRIES, m);
            LPROF_ADD(LP_CLASS + c, 1);
            LPROF_ADD(LP_CLASS_ENT + c, m);
            LPROF_ADD(LP_CLASS_CYC + c, t_w1 - t_list);
        }
#endif
    }
#if PJG_SEARCH_PROF
    // the comparison counts differ by lane; every other sum is warp-uniform
    for (int off = 16; off; off >>= 1) lp[LP_COUNT_PAIRS] += __shfl_xor_sync(FULL_MASK, lp[LP_COUNT_PAIRS], off);
    if (lane == 0)
        for (int i = 0; i < LP_NUM; i++)
            if (lp[i]) atomicAdd(&g_leaf_prof[i], lp[i]);
#endif
    if (lane == 0 && n_exact) atomicAdd(&counters[C_LEAF_EXACT], n_exact);
    if (lane == 0 && n_sorted) atomicAdd(&counters[C_LEAF_SORTED], n_sorted);
    if (lane == 0 && n_lists) atomicAdd(&counters[C_LEAF_LISTS], n_lists);
    if (lane == 0 && n_entries) atomicAdd(&counters[C_LEAF_ENTRIES], n_entries);
}

// ---------------------------------------------------------------------------
// k_leaf_part: tie-free lists by axis partitions, one warp per list.
//
// The three axis orders of the list are sorted once (bitmap over the
// structure's unique axis ranks, sort_segment); then every level takes, in
// each node, the first n/2 entries of the split axis's order as the left
// child (the n/2 smallest: the same sets k_leaf_order's ranks give), marks
// them in one ballot pass over that order, and moves the other two orders
// to their children by a stable partition (one ballot prefix a 32-entry
// chunk).  O(m / 32) warp steps a level instead of the rank method's
// O(m n / 32).  A tie at a median boundary (equal strict-lower ranks on both
// sides of position n/2) hands the list on to k_leaf_sorted, which replays
// qselect there.  Leaves and block boxes are written from the cached atom
// indices, each 32-leaf chunk's boxes reduced in registers.

template <int CAP>
struct PartWarp {
    uint16_t S[4][CAP];   // the three axis orders and a spare (candidate indices)
    uint16_t lr[3][CAP];  // strict-lower axis ranks by candidate index (low 16
                          // bits: a false tie only hands the list on)
    int32_t atom[CAP];    // structure atom of each candidate index
    union {
        uint32_t ur[CAP];  // unique ranks of the axis being sorted
        struct {
            uint32_t seg[CAP];   // node of each position: lo | n << 16
            uint16_t base[CAP];  // at a node's first position: left members
                                 // of the nodes before it
            uint8_t flag[CAP];   // candidate goes to the left child
        } lv;
    } u;
    uint32_t bits[LEAF_SORT_WORDS];
    uint16_t wpre[LEAF_SORT_WORDS];
};

// sort_segment's bitmap sort on a PartWarp: S_out[0..m) = candidate indices
// 0..m-1 (keys L.u.ur) in key order; false when a key repeats
template <int CAP>
__device__ bool part_sort(PartWarp<CAP> &L, uint16_t *S_out, int m, int natoms) {
    const int lane = lane_id();
    constexpr int WB = 32 * LEAF_SORT_WORDS;
    int placed = 0;
    for (int wb = 0; wb < natoms; wb += WB) {
        const int nwords = min(LEAF_SORT_WORDS, (natoms - wb + 31) >> 5);
        for (int q = lane; q < nwords; q += 32) L.bits[q] = 0u;
        __syncwarp();
        for (int i = lane; i < m; i += 32) {
            const uint32_t u = L.u.ur[i] - (uint32_t)wb;
            if (u < (uint32_t)WB) atomicOr(&L.bits[u >> 5], 1u << (u & 31));
        }
        __syncwarp();
        int carry = placed;
        for (int w0 = 0; w0 < nwords; w0 += 32) {
            const int wd = w0 + lane;
            const int c = wd < nwords ? __popc(L.bits[wd]) : 0;
            int incl = c;
            for (int off = 1; off < 32; off <<= 1) {
                const int y = __shfl_up_sync(FULL_MASK, incl, off);
                if (lane >= off) incl += y;
            }
            if (wd < nwords) L.wpre[wd] = (uint16_t)(carry + incl - c);
            carry += __shfl_sync(FULL_MASK, incl, 31);
        }
        __syncwarp();
        for (int i = lane; i < m; i += 32) {
            const uint32_t u = L.u.ur[i] - (uint32_t)wb;
            if (u < (uint32_t)WB) {
                const int pos = L.wpre[u >> 5] + __popc(L.bits[u >> 5] & ((1u << (u & 31)) - 1u));
                if (pos < m) S_out[pos] = (uint16_t)i;
            }
        }
        __syncwarp();
        placed = carry;
    }
    return placed == m;
}

// Lists of at most take_max <= CAP entries without a median tie.  Longer
// lists go to fwd_list[0] (up to fwd_max[0] entries) or fwd_list[1] (up to
// fwd_max[1]) when given, else to k_leaf_sorted's worklists by size class
// (up to LEAF_SORTED_MAX) or k_leaf_exact's; tied lists likewise to the
// sorted or exact worklists.  count_lists: this instance counts the lists
// it is given (the first instance; the others see lists already counted).
template <int CAP, int WARPS>
__global__ void __launch_bounds__(WARPS * 32)
    k_leaf_part(ChunkView cv, int32_t n_sigs, const int32_t *count, const int64_t *offset,
                const int64_t *blk_offset, const int32_t *cand_atom, const int64_t *leaf_offset,
                int32_t *leaf_atom, float4 *leaf_xyz, float4 *blk_lo, float4 *blk_hi, int64_t *sorted_list,
                unsigned long long *sorted_count, int64_t list_cap, int64_t *exact_list,
                unsigned long long *exact_count, unsigned long long *counters, int take_max, const int64_t *work,
                const unsigned long long *n_work, int64_t *fwd_list0, unsigned long long *fwd_count0,
                int fwd_max0, int64_t *fwd_list1, unsigned long long *fwd_count1, int fwd_max1,
                int count_lists, uint8_t *part_ok) {
    extern __shared__ __align__(16) unsigned char part_smem[];
    PartWarp<CAP> &L = reinterpret_cast<PartWarp<CAP> *>(part_smem)[threadIdx.x >> 5];
    const int lane = lane_id();
    const unsigned lt = (1u << lane) - 1u;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t total = work ? (int64_t)*n_work : (int64_t)cv.n_structures * n_sigs;
    unsigned long long n_exact = 0, n_sorted = 0, n_lists = 0, n_entries = 0;
#if PJG_SEARCH_PROF
    unsigned long long lp[LP_NUM] = {};
#endif
    for (int64_t item = warp; item < total; item += nwarps) {
        const int64_t w = work ? work[item] : item;
        const int m = count[w];
        if (m <= 0) continue;
        if (count_lists) {
            n_lists++;
            n_entries += (unsigned long long)m;
        }
        bool handoff = m > take_max;
        LPROF_T(t_list);
        if (handoff && fwd_list0 && m <= fwd_max0) {
            if (lane == 0) fwd_list0[atomicAdd(fwd_count0, 1ull)] = w;
            __syncwarp();
            continue;
        }
        if (handoff && fwd_list1 && m <= fwd_max1) {
            if (lane == 0) fwd_list1[atomicAdd(fwd_count1, 1ull)] = w;
            __syncwarp();
            continue;
        }
        const int s = (int)(w / n_sigs);
        const int64_t gbase = cv.atom_base[s];
        const int natoms = cv.atom_count[s];
        const int32_t *ca = cand_atom + offset[w];
        bool exact = false;
        if (!handoff) {
            // atoms, strict-lower ranks, x ranks; then the three axis orders
            LPROF_T(t_l0);
#pragma unroll 4
            for (int i = lane; i < m; i += 32) {
                const int a = ca[i];
                const int64_t g = gbase + a;
                L.atom[i] = a;
                L.lr[0][i] = (uint16_t)cv.lrank[g];
                L.lr[1][i] = (uint16_t)cv.lrank[cv.n_atoms + g];
                L.lr[2][i] = (uint16_t)cv.lrank[2 * cv.n_atoms + g];
                L.u.ur[i] = cv.urank[g];
            }
            __syncwarp();
            {
                LPROF_T(t_l1);
                LPROF_ADD(LP_CYC_LOAD, t_l1 - t_l0);
            }
            for (int a = 0; a < 3 && !exact; a++) {
                if (a > 0) {
                    LPROF_T(t_g0);
#pragma unroll 4
                    for (int i = lane; i < m; i += 32) L.u.ur[i] = cv.urank[a * cv.n_atoms + gbase + L.atom[i]];
                    __syncwarp();
                    LPROF_T(t_g1);
                    LPROF_ADD(LP_CYC_LOAD, t_g1 - t_g0);
                }
                LPROF_T(t_s0);
                // a repeated atom (never in a candidate list) goes to the
                // exact replay
                exact = !part_sort(L, L.S[a], m, natoms);
                LPROF_T(t_s1);
                LPROF_ADD(LP_CYC_SORT, t_s1 - t_s0);
                LPROF_ADD(LP_SORT_NODES, 1);
                LPROF_ADD(LP_SORT_WORDS, (natoms + 31) >> 5);
            }
        }
        LPROF_T(t_lv);
        if (!handoff && !exact) {
            for (int p = lane; p < m; p += 32) L.u.lv.seg[p] = (uint32_t)m << 16;
            __syncwarp();
            int cur0 = 0, cur1 = 1, cur2 = 2, spare = 3;
            int levels = 0;
            while ((1 << levels) < m) levels++;
            for (int d = 0; d < levels; d++) {
                const int a = d % 3;
                const uint16_t *Sa = L.S[a == 0 ? cur0 : a == 1 ? cur1 : cur2];
                const uint16_t *La = L.lr[a];
                // left members of every node from the split axis's order,
                // and the median-boundary tie check
                bool tie = false;
                int carry = 0;
#pragma unroll 2
                for (int p0 = 0; p0 < m; p0 += 32) {
                    const int p = p0 + lane;
                    const bool valid = p < m;
                    const uint32_t sg = valid ? L.u.lv.seg[p] : 0u;
                    const int lo = (int)(sg & 0xFFFFu), n = (int)(sg >> 16), k = n >> 1;
                    const int e = valid ? Sa[p] : 0;
                    const bool left = n >= 2 && p < lo + k;
                    if (valid) L.u.lv.flag[e] = (uint8_t)left;
                    if (n >= 2 && p == lo + k) tie |= La[Sa[p - 1]] == La[e];
                    const unsigned bal = __ballot_sync(FULL_MASK, left);
                    if (valid && p == lo) L.u.lv.base[p] = (uint16_t)(carry + __popc(bal & lt));
                    carry += __popc(bal);
                }
                if (__any_sync(FULL_MASK, tie)) {
                    handoff = true;
                    break;
                }
                __syncwarp();
                // the other two orders, stably partitioned within each node;
                // the second pass also moves every position to its child node
                for (int t = 1; t <= 2; t++) {
                    const int b = (a + t) % 3;
                    const int cb = b == 0 ? cur0 : b == 1 ? cur1 : cur2;
                    const uint16_t *src = L.S[cb];
                    uint16_t *dst = L.S[spare];
                    int fc = 0;
#pragma unroll 2
                    for (int p0 = 0; p0 < m; p0 += 32) {
                        const int p = p0 + lane;
                        const bool valid = p < m;
                        const int e = valid ? src[p] : 0;
                        const bool f = valid && L.u.lv.flag[e];
                        const unsigned bal = __ballot_sync(FULL_MASK, f);
                        const int Fp = fc + __popc(bal & lt);
                        fc += __popc(bal);
                        if (valid) {
                            uint32_t sg = L.u.lv.seg[p];
                            const int lo = (int)(sg & 0xFFFFu), n = (int)(sg >> 16), k = n >> 1;
                            int to = p;
                            if (n >= 2) {
                                const int lb = Fp - (int)L.u.lv.base[lo];  // left members before p in its node
                                to = f ? lo + lb : p + k - lb;
                                if (t == 2) sg = p < lo + k ? ((uint32_t)lo | ((uint32_t)k << 16))
                                                            : ((uint32_t)(lo + k) | ((uint32_t)(n - k) << 16));
                            }
                            dst[to] = (uint16_t)e;
                            if (t == 2) L.u.lv.seg[p] = sg;
                        }
                    }
                    __syncwarp();
                    if (b == 0) cur0 = spare;
                    else if (b == 1) cur1 = spare;
                    else cur2 = spare;
                    spare = cb;
                }
            }
            LPROF_T(t_lv1);
            LPROF_ADD(LP_CYC_COUNT, t_lv1 - t_lv);
            if (!handoff) {
                // leaves in reverse partition order (the query pops the right
                // subtree first) and the boxes of their CULL_BLK-leaf blocks
                const uint16_t *fin = L.S[cur0];
                const float4 *pts = cv.xyz32 + gbase;
                const int64_t lo_out = leaf_offset[w], bo = blk_offset[w];
                for (int r0 = 0; r0 < m; r0 += 32) {
                    const int r = r0 + lane;
                    const bool valid = r < m;
                    const int a = valid ? L.atom[fin[m - 1 - r]] : 0;
                    const float4 x = valid ? pts[a] : make_float4(0.f, 0.f, 0.f, 0.f);
                    if (valid) {
                        leaf_atom[lo_out + r] = a;
                        leaf_xyz[lo_out + r] = x;
                    }
                    float mnx = valid ? x.x : INFINITY, mny = valid ? x.y : INFINITY, mnz = valid ? x.z : INFINITY;
                    float mxx = valid ? x.x : -INFINITY, mxy = valid ? x.y : -INFINITY,
                          mxz = valid ? x.z : -INFINITY;
                    for (int off = CULL_BLK / 2; off; off >>= 1) {
                        mnx = fminf(mnx, __shfl_xor_sync(FULL_MASK, mnx, off));
                        mny = fminf(mny, __shfl_xor_sync(FULL_MASK, mny, off));
                        mnz = fminf(mnz, __shfl_xor_sync(FULL_MASK, mnz, off));
                        mxx = fmaxf(mxx, __shfl_xor_sync(FULL_MASK, mxx, off));
                        mxy = fmaxf(mxy, __shfl_xor_sync(FULL_MASK, mxy, off));
                        mxz = fmaxf(mxz, __shfl_xor_sync(FULL_MASK, mxz, off));
                    }
                    if ((lane & (CULL_BLK - 1)) == 0 && valid) {
                        blk_lo[bo + r / CULL_BLK] = make_float4(mnx, mny, mnz, 0.f);
                        blk_hi[bo + r / CULL_BLK] = make_float4(mxx, mxy, mxz, 0.f);
                    }
                }
                if (part_ok && lane == 0) part_ok[w] = 1;
                __syncwarp();
#if PJG_SEARCH_PROF
                {
                    LPROF_T(t_w1);
                    const int c = leaf_class(m);
                    LPROF_ADD(LP_CYC_WRITE, t_w1 - t_lv1);
                    LPROF_ADD(LP_CYC_LIST, t_w1 - t_list);
                    LPROF_ADD(LP_LISTS, 1);
                    LPROF_ADD(LP_ENTRIES, m);
                    LPROF_ADD(LP_CLASS + c, 1);
                    LPROF_ADD(LP_CLASS_ENT + c, m);
                    LPROF_ADD(LP_CLASS_CYC + c, t_w1 - t_list);
                }
#endif
                continue;
            }
        }
        LPROF_ADD(LP_HANDED, 1);
        if (!exact && m <= LEAF_SORTED_MAX) {
            // size classes of k_leaf_sorted: up to 512, 1024, 2048 entries
            const int c = m <= 512 ? 0 : m <= 1024 ? 1 : 2;
            n_sorted++;
            if (lane == 0) sorted_list[c * list_cap + (int64_t)atomicAdd(&sorted_count[c], 1ull)] = w;
        } else {
            n_exact++;
            if (lane == 0) exact_list[atomicAdd(exact_count, 1ull)] = w;
        }
        __syncwarp();
    }
#if PJG_SEARCH_PROF
    if (lane == 0)
        for (int i = 0; i < LP_NUM; i++)
            if (lp[i]) atomicAdd(&g_leaf_prof[i], lp[i]);
#endif
    if (lane == 0 && n_exact) atomicAdd(&counters[C_LEAF_EXACT], n_exact);
    if (lane == 0 && n_sorted) atomicAdd(&counters[C_LEAF_SORTED], n_sorted);
    if (lane == 0 && n_lists) atomicAdd(&counters[C_LEAF_LISTS], n_lists);
    if (lane == 0 && n_entries) atomicAdd(&counters[C_LEAF_ENTRIES], n_entries);
}

// ---------------------------------------------------------------------------
// Lists with the same atoms share one kd leaf order.
//
// The candidate lists of one structure are built per template-atom
// signature, and different signatures often select the same atoms (an
// extra residue name with no atom of the listed name in it, the residue
// names in another order, ...).  A leaf order without a median tie depends
// only on the set of atoms (k_leaf_part's splits read nothing else), and
// any leaf order depends only on the candidate sequence, so each requested
// list is keyed by (structure, length, a hash of its atom set), the first
// list to claim a key is ordered, and every other list with that key takes
// the representative's leaves and blocks -- after checking that its
// sequence is the representative's, or that its set is and the
// representative was ordered without a tie.  Lists failing the check are
// ordered on their own.  Candidate lists never repeat an atom, so equal
// lengths and inclusion make equal sets.

__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    // the splitmix64 output function (Steele, Lea and Flood, 2014)
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

__global__ void k_list_keys(int32_t n_sigs, const int32_t *count, const int64_t *offset, const int32_t *cand_atom,
                            const int64_t *work, const unsigned long long *n_work, ListShare ls,
                            unsigned long long *counters) {
    const int lane = lane_id();
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t total = (int64_t)*n_work;
    unsigned long long n_lists = 0, n_entries = 0;
    // 32 consecutive items a warp: the lists hashed one after the other by
    // the whole warp, then every lane inserts its own list's key
    for (int64_t base = warp * 32; base < total; base += nwarps * 32) {
        const int64_t item = base + lane;
        const bool valid = item < total;
        const int64_t w = valid ? work[item] : 0;
        const int m = valid ? count[w] : 0;
        const int64_t off = valid ? offset[w] : 0;
        unsigned long long key = 0;
        const int nt = total - base < 32 ? (int)(total - base) : 32;
        for (int t = 0; t < nt; t++) {
            const int mt = __shfl_sync(FULL_MASK, m, t);
            const int64_t ot = __shfl_sync(FULL_MASK, off, t);
            const int32_t *ca = cand_atom + ot;
            // two order-independent sums of mixed atom indices
            unsigned long long h1 = 0, h2 = 0;
            for (int i = lane; i < mt; i += 32) {
                const unsigned long long a = (unsigned long long)(uint32_t)ca[i];
                h1 += mix64(a + 0x9e3779b97f4a7c15ull);
                h2 += mix64(a * 0xd6e8feb86659fd93ull + 0x632be59bd9b4e019ull);
            }
            for (int o = 16; o; o >>= 1) {
                h1 += __shfl_xor_sync(FULL_MASK, h1, o);
                h2 += __shfl_xor_sync(FULL_MASK, h2, o);
            }
            if (lane == t) key = h1 ^ ((h2 << 29) | (h2 >> 35));
        }
        if (valid) {
            key = mix64(key ^ ((unsigned long long)(w / n_sigs) << 40) ^ (unsigned long long)m) | 1ull;
            // linear probing, at most one lap (the table holds twice the
            // chunk's lists, so it never fills)
            int64_t sl = (int64_t)(key & (unsigned long long)ls.mask), found = -1;
            for (int64_t it = 0; it <= ls.mask; it++) {
                const unsigned long long prev = atomicCAS(&ls.key[sl], 0ull, key);
                if (prev == 0ull || prev == key) {
                    found = sl;
                    break;
                }
                sl = (sl + 1) & ls.mask;
            }
            if (found >= 0) atomicCAS(&ls.rep[found], -1, (int32_t)w);
            ls.slot[item] = (int32_t)found;
            n_lists++;
            n_entries += (unsigned long long)(m > 0 ? m : 0);
        }
    }
    for (int o = 16; o; o >>= 1) {
        n_lists += __shfl_xor_sync(FULL_MASK, n_lists, o);
        n_entries += __shfl_xor_sync(FULL_MASK, n_entries, o);
    }
    if (lane == 0 && n_lists) atomicAdd(&counters[C_LEAF_LISTS], n_lists);
    if (lane == 0 && n_entries) atomicAdd(&counters[C_LEAF_ENTRIES], n_entries);
}

__global__ void k_list_reps(const int64_t *work, const unsigned long long *n_work, ListShare ls) {
    const int lane = lane_id();
    const unsigned lt = (1u << lane) - 1u;
    const int64_t total = (int64_t)*n_work;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    // whole warps step through the items (warp-aggregated appends)
    for (int64_t i0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) & ~31ll; i0 < total; i0 += stride) {
        const int64_t item = i0 + lane;
        const bool valid = item < total;
        int64_t w = 0;
        int32_t r = -1;
        if (valid) {
            w = work[item];
            const int32_t sl = ls.slot[item];
            r = sl >= 0 ? ls.rep[sl] : -1;
        }
        const bool own = valid && (r < 0 || (int64_t)r == w);
        const bool dup = valid && !own;
        const unsigned mo = __ballot_sync(FULL_MASK, own), md = __ballot_sync(FULL_MASK, dup);
        unsigned long long bo = 0, bd = 0;
        if (lane == 0) {
            if (mo) bo = atomicAdd(&ls.n[0], (unsigned long long)__popc(mo));
            if (md) bd = atomicAdd(&ls.n[1], (unsigned long long)__popc(md));
        }
        bo = __shfl_sync(FULL_MASK, bo, 0);
        bd = __shfl_sync(FULL_MASK, bd, 0);
        if (own) ls.rep_work[bo + __popc(mo & lt)] = w;
        if (dup) ls.dup_work[bd + __popc(md & lt)] = (w << 32) | (int64_t)(uint32_t)r;
    }
}

template <int WARPS>
__global__ void __launch_bounds__(WARPS * 32)
    k_list_share(ChunkView cv, int32_t n_sigs, const int32_t *count, const int64_t *offset,
                 const int32_t *cand_atom, int64_t *leaf_offset, int64_t *blk_offset, ListShare ls,
                 unsigned long long *counters) {
    __shared__ uint32_t bits[WARPS][LEAF_SORT_WORDS];
    constexpr int WB = 32 * LEAF_SORT_WORDS;
    const int lane = lane_id();
    uint32_t *B = bits[threadIdx.x >> 5];
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t total = (int64_t)ls.n[1];
    unsigned long long n_shared = 0;
    // 32 consecutive duplicates a warp: each lane loads one's lengths and
    // offsets, then the warp checks them one after the other
    for (int64_t base = warp * 32; base < total; base += nwarps * 32) {
        const int64_t item = base + lane;
        int64_t w = 0, r = 0, ow = 0, orr = 0;
        int m = 0;
        bool same = false;
        if (item < total) {
            const int64_t v = ls.dup_work[item];
            w = v >> 32;
            r = (int64_t)(uint32_t)(v & 0xFFFFFFFFll);
            m = count[w];
            same = count[r] == m && (r / n_sigs) == (w / n_sigs);
            ow = offset[w];
            orr = offset[r];
        }
        const int nt = total - base < 32 ? (int)(total - base) : 32;
        bool verdict = false;
        for (int t = 0; t < nt; t++) {
            const int mt = __shfl_sync(FULL_MASK, m, t);
            bool st = __shfl_sync(FULL_MASK, same, t);
            if (!st) continue;
            const int64_t rt = __shfl_sync(FULL_MASK, r, t), wt = __shfl_sync(FULL_MASK, w, t);
            const int32_t *cw = cand_atom + __shfl_sync(FULL_MASK, ow, t);
            const int32_t *cr = cand_atom + __shfl_sync(FULL_MASK, orr, t);
            bool eq = true;
            for (int k = lane; k < mt; k += 32) eq &= cw[k] == cr[k];
            if (!__all_sync(FULL_MASK, eq)) {
                // the same set: every atom of w marked by r, one window of
                // the structure's atom indices at a time
                st = ls.part_ok[rt] != 0;
                const int natoms = cv.atom_count[(int)(wt / n_sigs)];
                for (int wb = 0; wb < natoms && st; wb += WB) {
                    const int nwords = min(LEAF_SORT_WORDS, (natoms - wb + 31) >> 5);
                    for (int q = lane; q < nwords; q += 32) B[q] = 0u;
                    __syncwarp();
                    for (int k = lane; k < mt; k += 32) {
                        const uint32_t u = (uint32_t)cr[k] - (uint32_t)wb;
                        if (u < (uint32_t)WB) atomicOr(&B[u >> 5], 1u << (u & 31));
                    }
                    __syncwarp();
                    bool in = true;
                    for (int k = lane; k < mt; k += 32) {
                        const uint32_t u = (uint32_t)cw[k] - (uint32_t)wb;
                        if (u < (uint32_t)WB) in &= ((B[u >> 5] >> (u & 31)) & 1u) != 0u;
                    }
                    st = __all_sync(FULL_MASK, in);
                    __syncwarp();
                }
            }
            if (lane == t) verdict = st;
        }
        if (item < total) {
            if (verdict) {
                leaf_offset[w] = leaf_offset[r];
                blk_offset[w] = blk_offset[r];
                n_shared++;
            }
        }
        const bool left = item < total && !verdict;
        const unsigned lm = __ballot_sync(FULL_MASK, left);
        if (lm) {
            unsigned long long b = 0;
            if (lane == 0) b = atomicAdd(&ls.n[2], (unsigned long long)__popc(lm));
            b = __shfl_sync(FULL_MASK, b, 0);
            if (left) ls.left_work[b + __popc(lm & ((1u << lane) - 1u))] = w;
        }
    }
    for (int o = 16; o; o >>= 1) n_shared += __shfl_xor_sync(FULL_MASK, n_shared, o);
    if (lane == 0 && n_shared) atomicAdd(&counters[C_LEAF_SHARED], n_shared);
}

// Exact replay for the lists k_leaf_order could not order by ranks (a tie
// at some median boundary, or a list too long for its shared buffer).
//
// One warp per list, the partitioned index array in shared memory.  Nodes
// of more than 32 points are split by the literal qselect_r sequence of
// median-of-3 pivots and Lomuto partitions, each partition computed by the
// whole warp: the "<= pivot" elements keep their order (prefix counts), and
// the ">" elements follow Lomuto's queue behaviour -- each ">" element is
// appended, each later "<=" element rotates the queue's front to its back --
// so every append is either a new element or a copy of append number r,
// resolved by pointer jumping.  Subtrees of at most 32 points are then
// handed one per lane and replayed sequentially.  Lists longer than
// EXACT_MAX use the sequential replay on one thread.

struct ExactShared {
    uint16_t *A;      // partitioned candidate positions
    double *key;      // axis value by candidate position (current node)
    uint16_t *X;      // "<=" elements of the partition in order
    uint16_t *VAL;    // queue appends (0xFFFF until resolved)
    uint16_t *PTR;    // append -> earlier append it copies
};

// One Lomuto partition of A[L0..R0] around A[piv] (moved to R0 first) by
// the whole warp; key[e] is element e's axis value ("<=" in the sense of
// axis_cmp: a NaN compares equal).  X, VAL and PTR are scratch of at least
// R0 - L0 entries.  Returns the pivot's final position.
template <typename KeyT>
__device__ int warp_lomuto(uint16_t *A, const KeyT *key, uint16_t *X, uint16_t *VAL, uint16_t *PTR, int L0, int R0,
                           int piv, unsigned long long *fallback) {
    struct {
        uint16_t *A, *X, *VAL, *PTR;
        const KeyT *key;
    } S{A, X, VAL, PTR, key};
    const int lane = lane_id();
    const unsigned lt = (1u << lane) - 1u;
    __syncwarp();
    if (lane == 0) {
        uint16_t t = S.A[R0];
        S.A[R0] = S.A[piv];
        S.A[piv] = t;
    }
    __syncwarp();
    const uint16_t P = S.A[R0];
    const KeyT pv = S.key[P];
    const int L = R0 - L0;
    int cf = 0, cpush = 0, crot = 0, capp = 0;
    for (int c0 = 0; c0 < L; c0 += 32) {
        const int i = c0 + lane;
        const bool valid = i < L;
        uint16_t xi = 0;
        bool f = false;
        if (valid) {
            xi = S.A[L0 + i];
            f = !(S.key[xi] > pv);
        }
        const unsigned mf = __ballot_sync(FULL_MASK, valid && f);
        const unsigned mp = __ballot_sync(FULL_MASK, valid && !f);
        const int push_before = cpush + __popc(mp & lt);
        const bool is_push = valid && !f;
        const bool is_rot = valid && f && push_before > 0;
        const unsigned mr = __ballot_sync(FULL_MASK, is_rot);
        const unsigned ma = mp | mr;
        if (valid && f) S.X[cf + __popc(mf & lt)] = xi;
        if (is_push || is_rot) {
            const int k = capp + __popc(ma & lt);
            if (is_push) {
                S.VAL[k] = xi;
                S.PTR[k] = (uint16_t)k;
            } else {
                S.VAL[k] = 0xFFFF;
                S.PTR[k] = (uint16_t)(crot + __popc(mr & lt));
            }
        }
        cf += __popc(mf);
        cpush += __popc(mp);
        crot += __popc(mr);
        capp += __popc(ma);
    }
    __syncwarp();
    // pointer jumping: at most log2(appends) + 1 rounds
    for (int round = 0; round < 20; round++) {
        bool open = false;
        for (int k = lane; k < capp; k += 32) {
            if (S.VAL[k] != 0xFFFF) continue;
            const int p = S.PTR[k];
            const uint16_t v = S.VAL[p];
            if (v != 0xFFFF) S.VAL[k] = v;
            else {
                S.PTR[k] = S.PTR[p];
                open = true;
            }
        }
        __syncwarp();
        if (!__any_sync(FULL_MASK, open)) break;
        if (round == 19 && lane == 0) atomicMax(fallback, 5ull);
    }
    const int C = cf, G = cpush, R = crot;
    for (int i = lane; i < C; i += 32) S.A[L0 + i] = S.X[i];
    if (G > 0) {
        for (int j = 1 + lane; j < G; j += 32) S.A[L0 + C + j] = S.VAL[R + j];
        if (lane == 0) S.A[R0] = S.VAL[R];
    }
    if (lane == 0) S.A[L0 + C] = P;
    __syncwarp();
    return L0 + C;
}

__device__ int warp_partition(const ExactShared &S, int L0, int R0, int piv, unsigned long long *fallback) {
    return warp_lomuto<double>(S.A, S.key, S.X, S.VAL, S.PTR, L0, R0, piv, fallback);
}

// sequential qselect_r on positions A[0..n) with their FP64 axis values in
// K[0], K[32], ... (one lane's interleaved slice, kept aligned with A
// through the swaps)
__device__ void lane_qselect(uint16_t *A, double *Kb, int n, int k) {
    auto K = [&](int i) -> double & { return Kb[32 * i]; };
    int left = 0, right = n - 1;
    for (;;) {
        if (left == right) return;
        int mid = (left + right + 1) / 2;
        double l = K(left), r = K(right), m = K(mid);
        int p;
        if ((axis_cmp(l, m) > 0) != (axis_cmp(l, r) > 0)) p = left;
        else if ((axis_cmp(m, l) < 0) != (axis_cmp(m, r) < 0)) p = mid;
        else p = right;
        uint16_t t = A[right];
        A[right] = A[p];
        A[p] = t;
        double tk = K(right);
        K(right) = K(p);
        K(p) = tk;
        double pv = K(right);
        int store = left;
        for (int i = left; i < right; i++) {
            if (axis_cmp(K(i), pv) <= 0) {
                uint16_t u = A[i];
                A[i] = A[store];
                A[store] = u;
                double uk = K(i);
                K(i) = K(store);
                K(store) = uk;
                store++;
            }
        }
        t = A[store];
        A[store] = A[right];
        A[right] = t;
        tk = K(store);
        K(store) = K(right);
        K(right) = tk;
        if (store == k) return;
        if (k < store) right = store - 1;
        else left = store + 1;
    }
}

// MAXN: longest list the instantiation keeps in shared memory; MINN: lists
// at or below it are left to the smaller instantiation
template <int MAXN, int MINN>
__global__ void k_leaf_exact(ChunkView cv, int32_t n_sigs, const int32_t *count, const int64_t *offset,
                             const int64_t *blk_offset, const int32_t *cand_atom, const int64_t *leaf_offset,
                             int32_t *leaf_atom, float4 *leaf_xyz, float4 *blk_lo, float4 *blk_hi,
                             const int64_t *exact_list, const unsigned long long *exact_count,
                             unsigned long long *counters) {
    extern __shared__ __align__(16) unsigned char esm[];
    const int lane = lane_id();
    constexpr int SMEM = MAXN * (8 + 2 * 4);
    static_assert(MAXN >= 1024, "the per-lane key slices need 8 KB");
    unsigned char *base = esm + (size_t)(threadIdx.x >> 5) * SMEM;
    ExactShared S;
    S.key = reinterpret_cast<double *>(base);
    S.A = reinterpret_cast<uint16_t *>(base + 8 * MAXN);
    S.X = S.A + MAXN;
    S.VAL = S.X + MAXN;
    S.PTR = S.VAL + MAXN;
    const int64_t total = (int64_t)*exact_count;
    int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = warp; i < total; i += nwarps) {
        const int64_t w = exact_list[i];
        const int m = count[w];
        if (m <= MINN || (m > MAXN && MAXN != EXACT_MAX)) continue;
        const int s = (int)(w / n_sigs);
        const int64_t o = offset[w];
        const int64_t lo = leaf_offset[w];
        const int32_t *ca = cand_atom + o;
        const double *xyz = cv.xyz64 + 3 * cv.atom_base[s];
        const float4 *pts = cv.xyz32 + cv.atom_base[s];
        if (m > MAXN) {
            // sequential replay on one lane, global scratch
            int32_t *perm = leaf_atom + lo;
            if (lane == 0) kd_exact(perm, m, ca, xyz);
            __syncwarp();
            for (int r = lane; r < m; r += 32) leaf_xyz[lo + r] = pts[ca[perm[m - 1 - r]]];
            __syncwarp();
            for (int r = lane; r < m / 2; r += 32) {
                int32_t x = perm[r], y = perm[m - 1 - r];
                perm[r] = ca[y];
                perm[m - 1 - r] = ca[x];
            }
            if (lane == 0 && (m & 1)) perm[m / 2] = ca[perm[m / 2]];
        } else {
            for (int p = lane; p < m; p += 32) S.A[p] = (uint16_t)p;
            __syncwarp();
            // large nodes: depth-first stack of (lo, n, axis), lane-uniform
            int st_lo[24], st_n[24], st_ax[24];
            int sp = 1;
            st_lo[0] = 0;
            st_n[0] = m;
            st_ax[0] = 0;
            // small subtrees collected for the lanes: (lo, n, axis) packed
            uint32_t small_mine[8];
            int n_small_mine = 0, n_small = 0;
            while (sp > 0) {
                sp--;
                const int lo = st_lo[sp], n = st_n[sp], ax = st_ax[sp];
                if (n <= 1) continue;
                if (n <= 32) {
                    // lane (n_small % 32) replays this subtree later
                    if ((n_small & 31) == lane && n_small_mine < 8)
                        small_mine[n_small_mine++] = (uint32_t)lo | ((uint32_t)n << 16) | ((uint32_t)ax << 24);
                    // children of nodes above 32 points have at least 16, so a
                    // list of EXACT_MAX points has at most 256 such subtrees
                    n_small++;
                    continue;
                }
                for (int p = lane; p < n; p += 32) S.key[S.A[lo + p]] = xyz[3 * (int64_t)ca[S.A[lo + p]] + ax];
                __syncwarp();
                const int k = n / 2;
                int left = 0, right = n - 1;
                while (left != right) {
                    const int L0 = lo + left, R0 = lo + right;
                    const int mid = (L0 + R0 + 1) / 2;
                    const double l = S.key[S.A[L0]], r = S.key[S.A[R0]], mm = S.key[S.A[mid]];
                    int piv;
                    if ((axis_cmp(l, mm) > 0) != (axis_cmp(l, r) > 0)) piv = L0;
                    else if ((axis_cmp(mm, l) < 0) != (axis_cmp(mm, r) < 0)) piv = mid;
                    else piv = R0;
                    const int store = warp_partition(S, L0, R0, piv, &counters[C_ERROR]) - lo;
                    if (store == k) break;
                    if (k < store) right = store - 1;
                    else left = store + 1;
                }
                const int nx = (ax + 1) % 3;
                st_lo[sp] = lo + k;
                st_n[sp] = n - k;
                st_ax[sp] = nx;
                sp++;
                st_lo[sp] = lo;
                st_n[sp] = k;
                st_ax[sp] = nx;
                sp++;
            }
            __syncwarp();
            // small subtrees, one lane each: the sequential recursion, with
            // the node's axis values staged in this lane's 32-slot slice of
            // the (now free) key array
            double *K = S.key + lane;  // element e of this lane's slice at K[32 e]
            for (int q = 0; q < n_small_mine; q++) {
                uint32_t v = small_mine[q];
                int slo = v & 0xFFFF, sn = (v >> 16) & 0xFF, sax = v >> 24;
                int ql[8], qn[8], qa[8];
                int qs = 1;
                ql[0] = slo;
                qn[0] = sn;
                qa[0] = sax;
                while (qs > 0) {
                    qs--;
                    int lo = ql[qs], n = qn[qs], ax = qa[qs];
                    if (n <= 1) continue;
                    int k = n / 2;
                    for (int e = 0; e < n; e++) K[32 * e] = xyz[3 * (int64_t)ca[S.A[lo + e]] + ax];
                    lane_qselect(S.A + lo, K, n, k);
                    int nx = (ax + 1) % 3;
                    ql[qs] = lo + k;
                    qn[qs] = n - k;
                    qa[qs] = nx;
                    qs++;
                    ql[qs] = lo;
                    qn[qs] = k;
                    qa[qs] = nx;
                    qs++;
                }
            }
            __syncwarp();
            if (n_small > 256 && lane == 0) atomicMax(&counters[C_ERROR], 4ull);
            for (int r = lane; r < m; r += 32) {
                int e = S.A[m - 1 - r];
                leaf_atom[lo + r] = ca[e];
                leaf_xyz[lo + r] = pts[ca[e]];
            }
        }
        __syncwarp();
        write_boxes(m, lo, leaf_xyz, blk_offset[w], blk_lo, blk_hi);
    }
}

// ---------------------------------------------------------------------------
// Axis ranks of every structure atom (once per structure set, at upload).
//
// For atom i and axis a: lrank = number of the structure's atoms whose
// coordinate on a is strictly smaller, so lranks compare exactly as the FP64
// coordinates do (equal coordinates share one); urank = number of atoms
// before i in (coordinate, index) order, a permutation of 0..n-1
// (coordinates are finite: pjg_structures_create rejects others).  One
// block per
// (structure, axis): the atoms are sorted in tiles of RANK_TILE in shared
// memory, each tile is stored, and every atom's ranks are sums of binary
// searches over the sorted tiles.

constexpr int RANK_TILE = 2048;
constexpr int RANK_THREADS = 512;

__device__ __forceinline__ unsigned long long order_key(double x) {
    if (x == 0.0) x = 0.0;  // -0 and +0 compare equal
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

__global__ void __launch_bounds__(RANK_THREADS)
    k_axis_ranks(const int64_t *atom_base, const int32_t *atom_count, const double *xyz64, int64_t n_atoms,
                 unsigned long long *tile_key, uint16_t *tile_idx, uint32_t *lrank, uint32_t *urank) {
    __shared__ unsigned long long key[RANK_TILE];
    __shared__ uint16_t idx[RANK_TILE];
    const int s = blockIdx.x, a = blockIdx.y;
    const int64_t b0 = atom_base[s];
    const int n = atom_count[s];
    const int tiles = (n + RANK_TILE - 1) / RANK_TILE;
    unsigned long long *gk = tile_key + a * n_atoms + b0;
    uint16_t *gi = tile_idx + a * n_atoms + b0;
    for (int t = 0; t < tiles; t++) {
        const int t0 = t * RANK_TILE, tn = min(RANK_TILE, n - t0);
        for (int i = threadIdx.x; i < RANK_TILE; i += blockDim.x) {
            if (i < tn) {
                key[i] = order_key(xyz64[3 * (b0 + t0 + i) + a]);
            } else {
                key[i] = ~0ull;
            }
            idx[i] = (uint16_t)i;
        }
        __syncthreads();
        // bitonic sort by (key, idx)
        for (int k = 2; k <= RANK_TILE; k <<= 1) {
            for (int j = k >> 1; j > 0; j >>= 1) {
                const int lj = __ffs(j) - 1;
                for (int q = threadIdx.x; q < RANK_TILE / 2; q += blockDim.x) {
                    const int i = ((q >> lj) << (lj + 1)) | (q & (j - 1));
                    const int l = i | j;
                    const bool asc = (i & k) == 0;
                    const unsigned long long ki = key[i], kl = key[l];
                    const uint16_t ii = idx[i], il = idx[l];
                    const bool gt = ki > kl || (ki == kl && ii > il);
                    if (gt == asc) {
                        key[i] = kl;
                        key[l] = ki;
                        idx[i] = il;
                        idx[l] = ii;
                    }
                }
                __syncthreads();
            }
        }
        for (int i = threadIdx.x; i < tn; i += blockDim.x) {
            gk[t0 + i] = key[i];
            gi[t0 + i] = idx[i];
        }
        __syncthreads();
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const unsigned long long ki = order_key(xyz64[3 * (b0 + i) + a]);
        const int ti = i / RANK_TILE;
        const uint16_t li = (uint16_t)(i % RANK_TILE);
        uint32_t lr = 0, ur = 0;
        for (int t = 0; t < tiles; t++) {
            const unsigned long long *tk = gk + t * RANK_TILE;
            const int tn = min(RANK_TILE, n - t * RANK_TILE);
            int lo = 0, hi = tn;
            while (lo < hi) {  // first key >= ki
                const int mid = (lo + hi) >> 1;
                if (tk[mid] < ki) lo = mid + 1;
                else hi = mid;
            }
            lr += lo;
            if (t < ti) {  // earlier atoms: equal keys come before i
                int l2 = lo, h2 = tn;
                while (l2 < h2) {
                    const int mid = (l2 + h2) >> 1;
                    if (tk[mid] <= ki) l2 = mid + 1;
                    else h2 = mid;
                }
                ur += l2;
            } else if (t == ti) {  // i's own tile: (key, index) order
                const uint16_t *tix = gi + t * RANK_TILE;
                int l2 = lo, h2 = tn;
                while (l2 < h2) {
                    const int mid = (l2 + h2) >> 1;
                    if (tk[mid] < ki || (tk[mid] == ki && tix[mid] < li)) l2 = mid + 1;
                    else h2 = mid;
                }
                ur += l2;
            } else {
                ur += lo;
            }
        }
        lrank[a * n_atoms + b0 + i] = lr;
        urank[a * n_atoms + b0 + i] = ur;
    }
}

// ---------------------------------------------------------------------------
// Sorted-axis leaf order (lists longer than the rank method's, or tied).
//
// One warp per list.  (1) Each axis order of the list comes from the atoms'
// unique axis ranks: set one bit per element in a bitmap over the
// structure's ranks (windows of SORT_WINDOW_BITS), prefix-count the words,
// and each element's position is the count of set bits below its own.
// Each element also gets its coordinate's dense rank within the list per
// axis (`run`), so that equal coordinates are exactly equal keys.  (2) The
// tree is split level by level: a node's left child is the first n/2
// entries of its range in the split axis's order, and the other orders are
// partitioned stably within each node by one prefix count per level.  (3)
// A node with a tie at its median boundary (equal keys on both sides of
// position n/2) keeps the elements qselect_r would leave on each side,
// which depends on the arrangement its ancestors' qselects leave behind:
// those ancestors and the node are replayed (median-of-3 pivots and Lomuto
// partitions, as in k_leaf_exact) on the arrangement array A, top down and
// each node at most once, and the node's children take their members from
// A.  Untied nodes need no arrangement: their children are the n/2
// smallest and the rest whatever the arrangement.  Lists whose tied nodes
// or replays exceed the small per-warp tables go to k_leaf_exact.

constexpr int SORT_WINDOW_WORDS = 512;
constexpr int SORT_WINDOW_BITS = 32 * SORT_WINDOW_WORDS;
constexpr int LEAF_MAX_TIED = 32;     // tied nodes per level
constexpr int LEAF_MAX_REPLAY = 64;   // replayed nodes per list

template <int M>
struct SortedWarp {
    uint16_t buf[4][M];  // the three axis orders and a spare (ping-pong)
    uint16_t run[3][M];  // dense coordinate rank of each element per axis
    union {
        struct {
            uint32_t bits[SORT_WINDOW_WORDS];
            uint16_t wpre[SORT_WINDOW_WORDS];  // set bits before each word
            uint32_t ur[M];                    // unique rank of each element
            uint32_t lr[M];                    // strict-lower rank of each element
        } so;
        struct {
            uint16_t base[M]; // left members of the nodes before a position's node
            uint16_t VAL[M];  // replay scratch
            uint16_t PTR[M];  // replay scratch
            uint16_t A[M];    // qselect arrangement of replayed nodes
            uint32_t seg[M];  // node of each position: lo | n << 16
            uint8_t flag[M];  // element goes to the left child
            uint32_t done[LEAF_MAX_REPLAY];
            uint16_t tied[LEAF_MAX_TIED];
        } sp;
    } u;
};

// qselect_r's k = n/2 selection on A[lo..lo+n) with keys K (see k_leaf_exact)
__device__ void warp_qselect(uint16_t *A, const uint16_t *K, uint16_t *X, uint16_t *VAL, uint16_t *PTR, int lo,
                             int n, unsigned long long *err) {
    const int k = n / 2;
    int left = 0, right = n - 1;
    while (left != right) {
        const int L0 = lo + left, R0 = lo + right;
        const int mid = (L0 + R0 + 1) / 2;
        const int l = K[A[L0]], r = K[A[R0]], mm = K[A[mid]];
        int piv;
        if ((l > mm) != (l > r)) piv = L0;
        else if ((mm < l) != (mm < r)) piv = mid;
        else piv = R0;
        const int store = warp_lomuto<uint16_t>(A, K, X, VAL, PTR, L0, R0, piv, err) - lo;
        if (store == k) break;
        if (k < store) right = store - 1;
        else left = store + 1;
    }
}

template <int M, int MINN, int WARPS>
__global__ void __launch_bounds__(WARPS * 32, 1)
    k_leaf_sorted(ChunkView cv, int32_t n_sigs, const int32_t *count, const int64_t *offset,
                  const int64_t *blk_offset, const int32_t *cand_atom, const int64_t *leaf_offset, int32_t *leaf_atom,
                  float4 *leaf_xyz, float4 *blk_lo, float4 *blk_hi, const int64_t *sorted_list,
                  const unsigned long long *sorted_count, int64_t *exact_list, unsigned long long *exact_count,
                  unsigned long long *counters) {
    extern __shared__ __align__(16) unsigned char sorted_smem[];
    SortedWarp<M> &L = reinterpret_cast<SortedWarp<M> *>(sorted_smem)[threadIdx.x >> 5];
    const int lane = lane_id();
    const unsigned lt = (1u << lane) - 1u;
    const int64_t total = (int64_t)*sorted_count;
    int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    unsigned long long n_exact = 0, n_replay = 0;
    for (int64_t i = warp; i < total; i += nwarps) {
        const int64_t w = sorted_list[i];
        const int m = count[w];
        if (m <= MINN || m > M) continue;
        const int s = (int)(w / n_sigs);
        const int64_t gbase = cv.atom_base[s];
        const int natoms = cv.atom_count[s];
        const int64_t o = offset[w];
        const int32_t *ca = cand_atom + o;

        // (1) axis orders and dense ranks
        bool complete = true;
        for (int a = 0; a < 3; a++) {
            const uint32_t *ur = cv.urank + a * cv.n_atoms + gbase;
            const uint32_t *lrk = cv.lrank + a * cv.n_atoms + gbase;
            uint16_t *Sa = L.buf[a];
#pragma unroll 4
            for (int e = lane; e < m; e += 32) {
                const int atom = ca[e];
                L.u.so.ur[e] = ur[atom];
                L.u.so.lr[e] = lrk[atom];
            }
            int placed = 0;
            for (int wb = 0; wb < natoms; wb += SORT_WINDOW_BITS) {
                const int nwords = min(SORT_WINDOW_WORDS, (natoms - wb + 31) >> 5);
                if (wb == 0)
                    for (int q = lane; q < nwords; q += 32) L.u.so.bits[q] = 0u;
                __syncwarp();
                for (int e = lane; e < m; e += 32) {
                    const uint32_t u = L.u.so.ur[e] - (uint32_t)wb;
                    if (u < (uint32_t)SORT_WINDOW_BITS) atomicOr(&L.u.so.bits[u >> 5], 1u << (u & 31));
                }
                __syncwarp();
                int carry = placed;
                for (int w0 = 0; w0 < nwords; w0 += 32) {
                    const int wd = w0 + lane;
                    const int c = wd < nwords ? __popc(L.u.so.bits[wd]) : 0;
                    int incl = c;
                    for (int off = 1; off < 32; off <<= 1) {
                        const int y = __shfl_up_sync(FULL_MASK, incl, off);
                        if (lane >= off) incl += y;
                    }
                    if (wd < nwords) L.u.so.wpre[wd] = (uint16_t)(carry - placed + incl - c);
                    carry += __shfl_sync(FULL_MASK, incl, 31);
                }
                __syncwarp();
                for (int e = lane; e < m; e += 32) {
                    const uint32_t u = L.u.so.ur[e] - (uint32_t)wb;
                    if (u < (uint32_t)SORT_WINDOW_BITS) {
                        const uint32_t word = L.u.so.bits[u >> 5];
                        Sa[placed + L.u.so.wpre[u >> 5] + __popc(word & ((1u << (u & 31)) - 1u))] = (uint16_t)e;
                    }
                }
                __syncwarp();
                for (int e = lane; e < m; e += 32) {
                    const uint32_t u = L.u.so.ur[e] - (uint32_t)wb;
                    if (u < (uint32_t)SORT_WINDOW_BITS) L.u.so.bits[u >> 5] = 0u;
                }
                __syncwarp();
                placed = carry;
            }
            if (placed != m) {  // an atom twice in the list: not a permutation
                complete = false;
                break;
            }
            // dense ranks: a new run wherever the strict-lower rank changes
            int c0 = 0;
            uint32_t prev = 0;
            for (int p0 = 0; p0 < m; p0 += 32) {
                const int p = p0 + lane;
                const int e = p < m ? Sa[p] : 0;
                const uint32_t l = p < m ? L.u.so.lr[e] : 0u;
                uint32_t before = __shfl_up_sync(FULL_MASK, l, 1);
                if (lane == 0) before = prev;
                const bool chg = p < m && (p == 0 || l != before);
                const unsigned mask = __ballot_sync(FULL_MASK, chg);
                if (p < m) L.run[a][e] = (uint16_t)(c0 + __popc(mask & (lt | (1u << lane))) - 1);
                c0 += __popc(mask);
                prev = __shfl_sync(FULL_MASK, l, 31);
            }
            __syncwarp();
        }

        // (2) level-by-level median splits
        bool bail = !complete;
        for (int p = lane; p < m; p += 32) L.u.sp.seg[p] = (uint32_t)m << 16;
        __syncwarp();
        int cur0 = 0, cur1 = 1, cur2 = 2, spare = 3;
        int nd = 0;
        int levels = 0;
        while ((1 << levels) < m) levels++;
        // flags (element goes left) and tied nodes of level `lev`, from the
        // axis order `Sx` and the node table; fused into the node update
        // of the level before
        int ntied = 0;
        auto mark_level = [&](int lev) {
            const int ax = lev % 3;
            const uint16_t *Sx = L.buf[ax == 0 ? cur0 : ax == 1 ? cur1 : cur2];
            const uint16_t *Rx = L.run[ax];
            ntied = 0;
            int left_before = 0;  // left positions of the level before this chunk
            for (int p0 = 0; p0 < m; p0 += 32) {
                const int p = p0 + lane;
                bool tie = false, left = false, start = false;
                int lo = 0;
                if (p < m) {
                    uint32_t sg = L.u.sp.seg[p];
                    lo = (int)(sg & 0xFFFFu);
                    int n = (int)(sg >> 16);
                    if (lev > 0 && n >= 2) {
                        // the node of level lev holding p (child of sg)
                        const int k = n >> 1;
                        if (p < lo + k) n = k;
                        else {
                            lo += k;
                            n -= k;
                        }
                        sg = (uint32_t)lo | ((uint32_t)n << 16);
                        L.u.sp.seg[p] = sg;
                    }
                    const int k = n >> 1;
                    const int e = Sx[p];
                    left = n >= 2 && p < lo + k;
                    start = p == lo;
                    L.u.sp.flag[e] = (uint8_t)left;
                    if (n >= 2 && p == lo + k) tie = Rx[Sx[p - 1]] == Rx[e];
                }
                const unsigned lm = __ballot_sync(FULL_MASK, left);
                if (start) L.u.sp.base[p] = (uint16_t)(left_before + __popc(lm & lt));
                __syncwarp();
                if (p < m && !start) L.u.sp.base[p] = L.u.sp.base[lo];
                left_before += __popc(lm);
                const unsigned mask = __ballot_sync(FULL_MASK, tie);
                if (tie) {
                    const int slot = ntied + __popc(mask & lt);
                    if (slot < LEAF_MAX_TIED) L.u.sp.tied[slot] = (uint16_t)lo;
                }
                ntied += __popc(mask);
            }
            __syncwarp();
        };
        if (levels > 0) mark_level(0);
        for (int d = 0; d < levels && !bail; d++) {
            const int a = d % 3;
            __syncwarp();
            if (ntied > LEAF_MAX_TIED) {
                bail = true;
                break;
            }
            for (int t = 0; t < ntied && !bail; t++) {
                const int tlo = L.u.sp.tied[t];
                const int tn = (int)(L.u.sp.seg[tlo] >> 16);
                int lj = 0, nj = m;
                for (int j = 0; j <= d; j++) {
                    if (j > 0) {
                        // child of the level j-1 node (lj, nj) holding tlo
                        const int k = nj >> 1;
                        if (tlo < lj + k) nj = k;
                        else {
                            lj += k;
                            nj -= k;
                        }
                    }
                    const uint32_t tag = ((uint32_t)j << 16) | (uint32_t)lj;
                    bool seen = false;
                    for (int q = lane; q < nd; q += 32) seen |= L.u.sp.done[q] == tag;
                    if (__any_sync(FULL_MASK, seen)) continue;
                    if (nd == LEAF_MAX_REPLAY) {
                        bail = true;
                        break;
                    }
                    if (nd == 0) {
                        for (int p = lane; p < m; p += 32) L.u.sp.A[p] = (uint16_t)p;
                        __syncwarp();
                    }
                    warp_qselect(L.u.sp.A, L.run[j % 3], L.buf[spare], L.u.sp.VAL, L.u.sp.PTR, lj, nj,
                                 &counters[C_ERROR]);
                    if (lane == 0) L.u.sp.done[nd] = tag;
                    nd++;
                    n_replay++;
                    __syncwarp();
                }
                if (bail) break;
                // the tied node's members from its qselect arrangement
                for (int p = tlo + lane; p < tlo + tn; p += 32)
                    L.u.sp.flag[L.u.sp.A[p]] = (uint8_t)(p < tlo + (tn >> 1));
                __syncwarp();
            }
            if (bail) break;
            // stable partition of the orders within each node
            bool bad = false;
            for (int b = 0; b < 3; b++) {
                if (b == a && ntied == 0) continue;
                const int cb = b == 0 ? cur0 : b == 1 ? cur1 : cur2;
                const uint16_t *src = L.buf[cb];
                uint16_t *dst = L.buf[spare];
                int carry = 0;
                for (int p0 = 0; p0 < m; p0 += 32) {
                    const int p = p0 + lane;
                    const bool valid = p < m;
                    const int e = valid ? src[p] : 0;
                    const bool f = valid && L.u.sp.flag[e];
                    const unsigned mask = __ballot_sync(FULL_MASK, f);
                    const int Fp = carry + __popc(mask & lt);
                    carry += __popc(mask);
                    if (valid) {
                        const uint32_t sg = L.u.sp.seg[p];
                        const int lo = (int)(sg & 0xFFFFu), n = (int)(sg >> 16);
                        int to = p;
                        if (n >= 2) {
                            // left members before p within its node
                            const int lb = Fp - (int)L.u.sp.base[p];
                            to = f ? lo + lb : p + (n >> 1) - lb;
                            // inside the node by construction (exactly n/2
                            // left members); checked all the same
                            if (to < lo || to >= lo + n) {
                                bad = true;
                                to = p;
                            }
                        }
                        dst[to] = (uint16_t)e;
                    }
                }
                __syncwarp();
                if (b == 0) cur0 = spare;
                else if (b == 1) cur1 = spare;
                else cur2 = spare;
                spare = cb;
            }
            if (__any_sync(FULL_MASK, bad)) {
                if (lane == 0) atomicMax(&counters[C_ERROR], 6ull);
                bail = true;
                break;
            }
            if (d + 1 < levels) mark_level(d + 1);
        }
        if (bail) {
            n_exact++;
            if (lane == 0) exact_list[atomicAdd(exact_count, 1ull)] = w;
            __syncwarp();
            continue;
        }
        write_leaves(L.buf[cur0], m, leaf_offset[w], ca, cv.xyz32 + gbase, leaf_atom, leaf_xyz, blk_offset[w], blk_lo,
                     blk_hi);
    }
    if (lane == 0 && n_exact) atomicAdd(&counters[C_LEAF_EXACT], n_exact);
    if (lane == 0 && n_replay) atomicAdd(&counters[C_LEAF_REPLAY], n_replay);
}

// Request list w (m entries) for kd leaf order: the first request moves it
// from state 0 to 1, reserves its place in the leaf arrays and queues it.
// List w is read in candidate order by some pair (its level 0): queue it
// for the fill (once).
__device__ __forceinline__ void request_fill(const LeafDemand &dm, int64_t w) {
    if (dm.fill_state && dm.fill_state[w] == 0 && atomicCAS(&dm.fill_state[w], 0, 1) == 0)
        dm.fill_work[atomicAdd(dm.n_fill, 1ull)] = w;
}

__device__ __forceinline__ void request_list(const LeafDemand &dm, int64_t w, int m) {
    if (dm.state[w] == 0 && atomicCAS(&dm.state[w], 0, 1) == 0) {
        dm.leaf_offset[w] = (int64_t)atomicAdd(dm.leaf_used, (unsigned long long)m);
        dm.work[atomicAdd(dm.n_work, 1ull)] = w;
    }
}

// Warp-wide forms of request_fill / request_list, called by every lane of
// the warp: the lists a lane wins (state 0 -> 1) get their leaf-array ranges
// and worklist places from one atomic add per warp.
__device__ __forceinline__ void request_fill_warp(const LeafDemand &dm, bool want, int64_t w) {
    const int lane = lane_id();
    const bool win =
        want && dm.fill_state && dm.fill_state[w] == 0 && atomicCAS(&dm.fill_state[w], 0, 1) == 0;
    const unsigned wm = __ballot_sync(FULL_MASK, win);
    if (!wm) return;
    unsigned long long b = 0;
    if (lane == 0) b = atomicAdd(dm.n_fill, (unsigned long long)__popc(wm));
    b = __shfl_sync(FULL_MASK, b, 0);
    if (win) dm.fill_work[b + __popc(wm & ((1u << lane) - 1u))] = w;
}

__device__ __forceinline__ void request_list_warp(const LeafDemand &dm, bool want, int64_t w, int m) {
    const int lane = lane_id();
    const bool win = want && dm.state[w] == 0 && atomicCAS(&dm.state[w], 0, 1) == 0;
    const unsigned wm = __ballot_sync(FULL_MASK, win);
    if (!wm) return;
    const unsigned long long mm = win ? (unsigned long long)m : 0ull;
    unsigned long long incl = mm;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = __shfl_up_sync(FULL_MASK, incl, o);
        if (lane >= o) incl += y;
    }
    const unsigned long long tot = __shfl_sync(FULL_MASK, incl, 31);
    unsigned long long bo = 0, bw = 0;
    if (lane == 0) {
        bo = atomicAdd(dm.leaf_used, tot);
        bw = atomicAdd(dm.n_work, (unsigned long long)__popc(wm));
    }
    bo = __shfl_sync(FULL_MASK, bo, 0);
    bw = __shfl_sync(FULL_MASK, bw, 0);
    if (win) {
        dm.leaf_offset[w] = (int64_t)(bo + incl - mm);
        dm.work[bw + __popc(wm & ((1u << lane) - 1u))] = w;
    }
}

// Lists needed before the search starts: a pair with no empty candidate
// list reads the lists of levels 1, 2, ... in kd leaf order as its frontier
// reaches them; the lists of the first `max_level` levels are requested
// here (thread per pair, the level order of k_search), deeper ones by the
// search itself when a pair first reaches them.  Consecutive threads take
// consecutive templates of one structure.
__global__ void k_demand_levels(TemplateView tv, CandView cd, int32_t n_pairs, int32_t max_level, int32_t reorder,
                                LeafDemand dm) {
    constexpr int TOP = 8;  // levels requested through the warp-wide path
    const int lane = lane_id();
    const int T = tv.n_templates, G = cd.n_sigs;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) & ~31ll; base < n_pairs; base += stride) {
        const int64_t pair = base + lane;
        int n = 0, ab = 0;
        int64_t wb = 0;
        if (pair < n_pairs) {
            const int s = (int)(pair / T), t = (int)(pair % T);
            ab = tv.atom_begin[t];
            n = tv.atom_begin[t + 1] - ab;
            wb = (int64_t)s * G;
        }
        // this pair's plan: levels 0..levels (-1: none) of atoms k_i
        int levels = -1;
        bool per_thread = false;
        unsigned long long top[TOP];
#pragma unroll
        for (int i = 0; i < TOP; i++) top[i] = ~0ull;
        if (n == 1) {
            if (cd.count[wb + tv.sig[ab]] > 0) levels = 0;  // its only list, in candidate order
            top[0] = 0;
        } else if (n > 32) {
            per_thread = true;  // k_search_large: every list, below
        } else if (n >= 2) {
            // the (max_level + 1) smallest (length, index) keys, sorted in
            // registers
            bool empty = false;
            for (int k = 0; k < n; k++) {
                const int c = cd.count[wb + tv.sig[ab + k]];
                empty |= c == 0;
                unsigned long long key = ((unsigned long long)(uint32_t)c << 5) | (unsigned long long)k;
#pragma unroll
                for (int i = 0; i < TOP; i++) {
                    const unsigned long long lo = key < top[i] ? key : top[i];
                    key = key < top[i] ? top[i] : key;
                    top[i] = lo;
                }
            }
            if (!empty) {
                levels = min(n - 1, max_level);
                if (levels >= TOP) per_thread = true;
            }
        }
        if (dm.pair_cost && pair < n_pairs) {
            // estimated cost: the product of the two shortest list lengths
            // (a one-atom template: its list's length), as a power-of-two
            // bucket; 0 for a pair with nothing to search here
            unsigned long long cost = 0;
            if (n == 1 && levels == 0) cost = (unsigned long long)cd.count[wb + tv.sig[ab]];
            else if (n >= 2 && n <= 32 && levels >= 0) cost = (top[0] >> 5) * (top[1] >> 5);
            dm.pair_cost[pair] = (uint8_t)(cost ? min(63, 64 - __clzll((long long)cost)) : 0);
        }
        // levels 0..TOP-1, warp-wide (every lane takes every step)
#pragma unroll
        for (int i = 0; i < TOP; i++) {
            const bool want = !per_thread && i <= levels;
            const int k = !want ? 0 : (reorder ? (int)(top[i] & 31ull) : i);
            const int64_t w = want ? wb + tv.sig[ab + k] : 0;
            if (i == 0) request_fill_warp(dm, want, w);
            else request_list_warp(dm, want, w, !want ? 0 : reorder ? (int)(top[i] >> 5) : cd.count[w]);
        }
        if (!per_thread) continue;
        if (n > 32) {
            // every list but the level-0 one, before the search (those pairs
            // never suspend); the level-0 atom has the smallest (length,
            // index)
            bool empty = false;
            int best = INT_MAX, best_k = 0;
            for (int k = 0; k < n; k++) {
                const int c = cd.count[wb + tv.sig[ab + k]];
                if (c == 0) empty = true;
                if (c < best) {
                    best = c;
                    best_k = k;
                }
            }
            if (empty) continue;
            const int k0 = reorder ? best_k : 0;
            for (int k = 0; k < n; k++) {
                const int64_t w = wb + tv.sig[ab + k];
                if (k != k0) request_list(dm, w, cd.count[w]);
                else request_fill(dm, w);
            }
        } else {
            // more levels than the register list holds: each atom's rank
            // from the keys below its own
            for (int k = 0; k < n; k++) {
                const int64_t w = wb + tv.sig[ab + k];
                const int c = cd.count[w];
                int rank = k;
                if (reorder) {
                    rank = 0;
                    for (int j = 0; j < n; j++) {
                        const int cj = cd.count[wb + tv.sig[ab + j]];
                        rank += (cj < c || (cj == c && j < k)) ? 1 : 0;
                    }
                }
                if (rank == 0) request_fill(dm, w);
                else if (rank <= max_level) request_list(dm, w, c);
            }
        }
    }
}

// Costliest pairs first.  Pass 1: a histogram of the pairs' cost buckets.
__global__ void k_cost_hist(int32_t n_pairs, const uint8_t *cost, unsigned long long *bins) {
    __shared__ unsigned int h[64];
    for (int i = threadIdx.x; i < 64; i += blockDim.x) h[i] = 0;
    __syncthreads();
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n_pairs; p += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(&h[cost[p]], 1u);
    __syncthreads();
    for (int i = threadIdx.x; i < 64; i += blockDim.x)
        if (h[i]) atomicAdd(&bins[i], (unsigned long long)h[i]);
}

// Pass 2: the threshold (the highest bucket at which the pairs of that
// bucket and above pass `target`; the pairs above it are heavy), then each
// heavy pair flagged and listed (bins[64]: their count).
__global__ void k_heavy_list(int32_t n_pairs, const uint8_t *cost, unsigned long long *bins, int64_t target,
                             uint8_t *heavy_flag, int32_t *heavy) {
    __shared__ int thr;
    if (threadIdx.x == 0) {
        unsigned long long acc = 0;
        int b = 63;
        for (; b > 0; b--) {
            acc += bins[b];
            if (acc > (unsigned long long)target) break;
        }
        thr = b;  // b == 0: every pair with a cost fits under the target
    }
    __syncthreads();
    const int lane = lane_id();
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t p0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) & ~31ll; p0 < n_pairs; p0 += stride) {
        const int64_t p = p0 + lane;
        const bool hv = p < n_pairs && cost[p] > thr;
        if (p < n_pairs) heavy_flag[p] = hv ? 1 : 0;
        const unsigned m = __ballot_sync(FULL_MASK, hv);
        if (m) {
            unsigned long long b = 0;
            if (lane == 0) b = atomicAdd(&bins[64], (unsigned long long)__popc(m));
            b = __shfl_sync(FULL_MASK, b, 0);
            if (hv) heavy[b + __popc(m & ((1u << lane) - 1u))] = (int32_t)p;
        }
    }
}

__global__ void k_mark_ordered(LeafDemand dm) {
    const int64_t n = (int64_t)*dm.n_work;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dm.state[dm.work[i]] = 2;
}

__global__ void k_block_counts(int64_t n, const int32_t *count, int32_t *nblk) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) nblk[i] = (count[i] + CULL_BLK - 1) / CULL_BLK;
}

// ---------------------------------------------------------------------------
// Superposition: warp per complete assignment.  Lanes hold the atom pairs
// (molecule atom, template atom) in template order, the warp reduces the
// centroids, the squared norms and the 3x3 cross-covariance S in FP64, and
// lane 0 solves the 4x4 quaternion eigenproblem: the largest root of the
// characteristic polynomial of Horn's key matrix by Newton's method from
// the upper bound (sumA + sumB)/2, the quaternion from the adjugate of
// (K - lambda I).  rmsd = sqrt(max(sumA + sumB - 2 lambda, 0) / n) and R
// maps molecule coordinates onto the template frame, as
// Superposition_rmsd / Superposition_rotation do.

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(FULL_MASK, v, o);
    return v;
}

__device__ double det3(double a, double b, double c, double d, double e, double f, double g, double h,
                       double i) {
    return a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g);
}

__device__ double det4(const double K[4][4]) {
    double d = 0.0;
    for (int c = 0; c < 4; c++) {
        int c0 = c == 0 ? 1 : 0;
        int c1 = c <= 1 ? 2 : 1;
        int c2 = c <= 2 ? 3 : 2;
        double minor = det3(K[1][c0], K[1][c1], K[1][c2], K[2][c0], K[2][c1], K[2][c2], K[3][c0],
                            K[3][c1], K[3][c2]);
        d += ((c & 1) ? -1.0 : 1.0) * K[0][c] * minor;
    }
    return d;
}

// 4x4 symmetric Jacobi: largest eigenvalue and its eigenvector.  Used when
// the top two eigenvalues of the key matrix are close (Newton's root of the
// characteristic polynomial then loses accuracy, and the adjugate
// eigenvector degenerates); Jacobi's eigenvalues are accurate to
// eps * |K| whatever the gap.
__device__ double jacobi4_top(double A[4][4], double v[4]) {
    double V[4][4];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) V[i][j] = i == j ? 1.0 : 0.0;
    double scale = 0.0;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) scale = fmax(scale, fabs(A[i][j]));
    for (int sweep = 0; sweep < 50; sweep++) {
        double off = 0.0;
        for (int p = 0; p < 4; p++)
            for (int q = p + 1; q < 4; q++) off += fabs(A[p][q]);
        if (off <= 1e-17 * scale) break;
        for (int p = 0; p < 3; p++)
            for (int q = p + 1; q < 4; q++) {
                if (A[p][q] == 0.0) continue;
                double theta = (A[q][q] - A[p][p]) / (2.0 * A[p][q]);
                double tt = 1.0 / (fabs(theta) + sqrt(theta * theta + 1.0));
                if (theta < 0) tt = -tt;
                double cc = 1.0 / sqrt(tt * tt + 1.0), ss = tt * cc;
                for (int r = 0; r < 4; r++) {
                    double arp = A[r][p], arq = A[r][q];
                    A[r][p] = cc * arp - ss * arq;
                    A[r][q] = ss * arp + cc * arq;
                }
                for (int r = 0; r < 4; r++) {
                    double apr = A[p][r], aqr = A[q][r];
                    A[p][r] = cc * apr - ss * aqr;
                    A[q][r] = ss * apr + cc * aqr;
                }
                for (int r = 0; r < 4; r++) {
                    double vrp = V[r][p], vrq = V[r][q];
                    V[r][p] = cc * vrp - ss * vrq;
                    V[r][q] = ss * vrp + cc * vrq;
                }
            }
    }
    int best = 0;
    for (int i = 1; i < 4; i++)
        if (A[i][i] > A[best][best]) best = i;
    for (int i = 0; i < 4; i++) v[i] = V[i][best];
    return A[best][best];
}

__device__ void key_matrix(const double S[9], double K[4][4]) {
    const double Sxx = S[0], Sxy = S[1], Sxz = S[2], Syx = S[3], Syy = S[4], Syz = S[5], Szx = S[6],
                 Szy = S[7], Szz = S[8];
    K[0][0] = Sxx + Syy + Szz; K[0][1] = Syz - Szy; K[0][2] = Szx - Sxz; K[0][3] = Sxy - Syx;
    K[1][0] = Syz - Szy; K[1][1] = Sxx - Syy - Szz; K[1][2] = Sxy + Syx; K[1][3] = Szx + Sxz;
    K[2][0] = Szx - Sxz; K[2][1] = Sxy + Syx; K[2][2] = -Sxx + Syy - Szz; K[2][3] = Syz + Szy;
    K[3][0] = Sxy - Syx; K[3][1] = Szx + Sxz; K[3][2] = Syz + Szy; K[3][3] = -Sxx - Syy + Szz;
}

// Largest eigenvalue of the key matrix: Newton on its characteristic
// polynomial l^4 + c2 l^2 + c1 l + c0 (c2 = -2 |S|^2, c1 = -8 det S,
// c0 = det K) from the upper bound E0 = (sumA + sumB) / 2.  The root's
// error is about eps * lambda^2 / gap; when P'(lambda) shows a gap below
// 1e-4 lambda, *close is set and the caller solves K by Jacobi instead.
__device__ double key_lambda(const double S[9], const double K[4][4], double E0, bool *close) {
    double fro = 0.0;
    for (int i = 0; i < 9; i++) fro += S[i] * S[i];
    const double c2 = -2.0 * fro;
    const double c1 = -8.0 * det3(S[0], S[1], S[2], S[3], S[4], S[5], S[6], S[7], S[8]);
    const double c0 = det4(K);
    double lam = E0;
    for (int it = 0; it < 60; it++) {
        double l2 = lam * lam;
        double P = (l2 + c2) * l2 + c1 * lam + c0;
        double dP = 4.0 * l2 * lam + 2.0 * c2 * lam + c1;
        if (dP == 0.0) break;
        double step = P / dP;
        lam -= step;
        if (fabs(step) <= 1e-14 * fabs(lam) + 1e-300) break;
    }
    double l2 = lam * lam;
    double dP = 4.0 * l2 * lam + 2.0 * c2 * lam + c1;
    *close = fabs(dP) < 4e-4 * fabs(l2 * lam);
    return lam;
}

__device__ __forceinline__ double rmsd_from_lambda(double E0, double lam, int n) {
    double r2 = 2.0 * (E0 - lam) / (double)n;
    return sqrt(r2 > 0.0 ? r2 : 0.0);
}

__device__ void quaternion_fit(const double S[9], double E0, int n, double *rmsd, double R[9], bool *bad) {
    double K[4][4];
    key_matrix(S, K);
    bool close = false;
    double lam = key_lambda(S, K, E0, &close);
    double best[4] = {0, 0, 0, 0}, bestn = -1.0;
    if (close) {
        double A[4][4];
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++) A[i][j] = K[i][j];
        lam = jacobi4_top(A, best);
        bestn = best[0] * best[0] + best[1] * best[1] + best[2] * best[2] + best[3] * best[3];
    }
    *rmsd = rmsd_from_lambda(E0, lam, n);
    // eigenvector: largest column of adj(K - lam I)
    double A[4][4];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) A[i][j] = K[i][j] - (i == j ? lam : 0.0);
    for (int col = 0; col < 4 && !close; col++) {
        double v[4];
        for (int row = 0; row < 4; row++) {
            // cofactor C[col][row] of A (adjugate column `col`)
            int r0 = col == 0 ? 1 : 0, r1 = col <= 1 ? 2 : 1, r2i = col <= 2 ? 3 : 2;
            int k0 = row == 0 ? 1 : 0, k1 = row <= 1 ? 2 : 1, k2 = row <= 2 ? 3 : 2;
            double m = det3(A[r0][k0], A[r0][k1], A[r0][k2], A[r1][k0], A[r1][k1], A[r1][k2], A[r2i][k0],
                            A[r2i][k1], A[r2i][k2]);
            v[row] = ((row + col) & 1) ? -m : m;
        }
        double nn = v[0] * v[0] + v[1] * v[1] + v[2] * v[2] + v[3] * v[3];
        if (nn > bestn) {
            bestn = nn;
            for (int i = 0; i < 4; i++) best[i] = v[i];
        }
    }
    double scale = 0.0;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) scale = fmax(scale, fabs(K[i][j]));
    if (!close && !(bestn > 1e-24 * scale * scale * scale * scale * scale * scale)) {
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++) A[i][j] = K[i][j];
        jacobi4_top(A, best);
        bestn = best[0] * best[0] + best[1] * best[1] + best[2] * best[2] + best[3] * best[3];
    }
    double inv = 1.0 / sqrt(bestn);
    double q0 = best[0] * inv, q1 = best[1] * inv, q2 = best[2] * inv, q3 = best[3] * inv;
    R[0] = q0 * q0 + q1 * q1 - q2 * q2 - q3 * q3;
    R[1] = 2.0 * (q1 * q2 - q0 * q3);
    R[2] = 2.0 * (q1 * q3 + q0 * q2);
    R[3] = 2.0 * (q1 * q2 + q0 * q3);
    R[4] = q0 * q0 - q1 * q1 + q2 * q2 - q3 * q3;
    R[5] = 2.0 * (q2 * q3 - q0 * q1);
    R[6] = 2.0 * (q1 * q3 - q0 * q2);
    R[7] = 2.0 * (q2 * q3 + q0 * q1);
    R[8] = q0 * q0 - q1 * q1 - q2 * q2 + q3 * q3;
    // the reference's rotation formula divides by the singular values of the
    // covariance and is undefined for fewer than three atom pairs
    *bad = n < 3;
}

// Centroids, centred covariance S = sum a b^T and E0 = (|a|^2 + |b|^2) / 2
// of one assignment, by one thread (sums in template atom order); atom(k)
// is the molecule atom matched to template atom k.
template <typename AtomOf>
__device__ __forceinline__ void lane_covariance_by(int n, AtomOf atom, const double *xyz, const double *tpos,
                                                   double ca[3], double cb[3], double S[9], double *E0) {
    for (int d = 0; d < 3; d++) ca[d] = cb[d] = 0.0;
    for (int k = 0; k < n; k++)
        for (int d = 0; d < 3; d++) {
            ca[d] += xyz[3 * (int64_t)atom(k) + d];
            cb[d] += tpos[3 * k + d];
        }
    for (int d = 0; d < 3; d++) {
        ca[d] /= (double)n;
        cb[d] /= (double)n;
    }
    double sumA = 0, sumB = 0;
    for (int q = 0; q < 9; q++) S[q] = 0.0;
    for (int k = 0; k < n; k++) {
        double a[3], b[3];
        for (int d = 0; d < 3; d++) {
            a[d] = xyz[3 * (int64_t)atom(k) + d] - ca[d];
            b[d] = tpos[3 * k + d] - cb[d];
        }
        sumA += a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
        sumB += b[0] * b[0] + b[1] * b[1] + b[2] * b[2];
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) S[3 * r + c] += a[r] * b[c];
    }
    *E0 = 0.5 * (sumA + sumB);
}

__device__ void lane_covariance(int n, const int32_t *atoms, const double *xyz, const double *tpos, double ca[3],
                                double cb[3], double S[9], double *E0) {
    lane_covariance_by(n, [&](int k) { return atoms[k]; }, xyz, tpos, ca, cb, S, E0);
}

// RMSD of one assignment computed by a single thread, used where a lane
// needs the value while searching (the same arithmetic as k_superpose).
template <typename AtomOf>
__device__ double lane_rmsd_by(int n, AtomOf atom, const double *xyz, const double *tpos) {
    double ca[3], cb[3], S[9], E0;
    lane_covariance_by(n, atom, xyz, tpos, ca, cb, S, &E0);
    double K[4][4];
    key_matrix(S, K);
    bool close = false;
    double lam = key_lambda(S, K, E0, &close);
    if (close) {
        double v[4];
        lam = jacobi4_top(K, v);
    }
    return rmsd_from_lambda(E0, lam, n);
}

__device__ double lane_rmsd(int n, const int32_t *atoms, const double *xyz, const double *tpos) {
    return lane_rmsd_by(n, [&](int k) { return atoms[k]; }, xyz, tpos);
}

// ---------------------------------------------------------------------------
// Search: warp per (structure, template) pair.
//
// The reference's Scanner_next is a depth-first backtracking over levels,
// level l taking template atom order[l] (order = identity, or sorted by
// candidate-list length when reorder is on, patches/Scanner.c.patch:97-108,
// 179-195).  Its stream of complete assignments is ordered
// lexicographically by (index in the level-0 list, kd leaf rank at level 1,
// ..., kd leaf rank at level n-1).  Here each level keeps a tile of partial
// assignments (entries = position in the level's list + index of the
// parent entry one level up); a tile is expanded against the next level's
// list in (parent, leaf rank) order with ballot + popc compaction, and a
// child tile is fully processed before its parent tile continues (depth
// first over tiles, breadth first inside a tile), which reproduces that
// order.
//
// Two expansion modes per level.  Block mode (lists of sa.block_min (64)
// or more): one parent at a time; its chain of atoms, key bits and FP32
// annulus bounds sit in shared memory and are read by all lanes as
// broadcasts; the parent's join box (intersection of its annulus boxes)
// culls whole blocks of CULL_BLK consecutive leaves by their bounding boxes, the
// leaves of the surviving blocks inside the join box are queued, and the
// full tests run on batches of 32 queued leaves.  Product mode (shorter
// lists): lanes take consecutive (parent, candidate) positions of the
// flattened product, so a warp step covers several parents.

struct PairState {
    int64_t lvl_off[32];
    int64_t blk_off[32];
    int32_t lvl_cnt[32];
    int32_t tkey[32];
    int32_t order[32];
    int32_t F[32];
    int32_t cnt[32];
    int32_t par[32];
    int32_t cnd[32];
    int32_t tile[32];
    // chain of the parent being expanded in block mode
    float4 cxyz[32];
    float4 cthr[32];
    int32_t cpos[32];
    // join box of the chain below the parent's level, and the parent index
    // (one level up) that chain belongs to
    float pbox[6];
    int32_t chain_gp;
    // block mode: leaves inside the parent's join box awaiting the full test
    float4 qxyz[64];
    int32_t qpos[64];
    // statistics of this warp's pairs (C_PAIRS .. C_BYTES_EXP), added to the
    // global counters once, when the warp exits
    unsigned long long acc[C_BYTES_EXP + 1];
};

size_t search_state_bytes() { return (sizeof(PairState) + 15) & ~size_t(15); }

template <typename PosT>
struct __align__(4) Entry {
    PosT pos;
    uint16_t parent;
};

// Exact FP64 annulus test of the reference (_Annulus_po,
// patches/Annulus.h.patch:54-68) plus the point-in-box test of the same
// annulus (its kd query box, patches/Annulus.c.patch:133-137).
__device__ __forceinline__ bool annulus64(const double *c, const double *x, const AnnulusParam &P,
                                          bool *in_box) {
    double sum = 0.0;
    for (int i = 0; i < 3; i++) {
        double t = __dsub_rn(c[i], x[i]);
        sum = __dadd_rn(sum, __dmul_rn(t, t));
    }
    bool inside = !(sum < P.a2 || sum > P.b2);
    bool ib = true;
    for (int i = 0; i < 3; i++) {
        if (x[i] < __dsub_rn(c[i], P.b) || x[i] > __dadd_rn(c[i], P.b)) ib = false;
    }
    *in_box = ib;
    return inside;
}

// The kd query prunes an internal node whose bounding box misses the join
// box B (intersection of the annulus boxes, Join_computeBox,
// patches/Join.c.patch:154-190; _Box_ro, patches/Box.h.patch:68-79).  A
// point inside every annulus box is never pruned; for a point that passes
// the annulus tests but lies outside B (possible only within rounding of a
// box face) walk the implicit tree to its leaf as the reference would.
__device__ __noinline__ bool kd_path_reaches(const int32_t *leaf_atom, int m, int rank, const double *xyz,
                                             const double *Bmin, const double *Bmax) {
    int q = m - 1 - rank;
    int lo = 0, hi = m;
    while (hi - lo > 1) {
        double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int r = m - hi; r < m - lo; r++) {
            const double *p = xyz + 3 * (int64_t)leaf_atom[r];
            for (int i = 0; i < 3; i++) {
                mn[i] = mn[i] < p[i] ? mn[i] : p[i];
                mx[i] = mx[i] > p[i] ? mx[i] : p[i];
            }
        }
        for (int i = 0; i < 3; i++)
            if (mn[i] > Bmax[i] || Bmin[i] > mx[i]) return false;
        int split = (hi - lo) / 2;
        if (q < lo + split) hi = lo + split;
        else lo = lo + split;
    }
    return true;
}

// TessTemplate_check (patches/TessTemplate.c.patch:101-155) for the newest
// atom against one earlier level, on packed (resSeq << 8 | chainID2) keys.
__device__ __forceinline__ bool check_pair(int32_t kj, int32_t kn, int32_t tj, int32_t tn, int ignore) {
    bool same_chain = (kj & 0xFF) == (kn & 0xFF);
    bool tsame_chain = (tj & 0xFF) == (tn & 0xFF);
    if (ignore == 0) {
        if (same_chain != tsame_chain) return false;
        if (!same_chain) return true;
    }
    bool same_res = (kj >> 8) == (kn >> 8);
    bool tsame_res = (tj >> 8) == (tn >> 8);
    if (same_res != tsame_res) return false;
    if (ignore != 2 && same_res && !same_chain) return false;
    return true;
}

// FP64 decision for one candidate whose FP32 test was inconclusive against
// at least one chain atom (`exact_mask`), or for every chain atom in FP64
// mode: the reference's annulus arithmetic, then the kd path check when the
// point lies outside an annulus box.
__device__ __noinline__ bool decide_fp64(unsigned exact_mask, int lev, const int32_t *atoms, int32_t an,
                                         const double *xyz, const AnnulusParam *prm, const int32_t *order,
                                         int n, int qn, const int32_t *leaf_atom_list, int mc, int cr) {
    bool need_path = false;
    const double *x = xyz + 3 * (int64_t)an;
    for (int j = 0; j <= lev; j++) {
        if (!((exact_mask >> j) & 1u)) continue;
        bool inb;
        if (!annulus64(xyz + 3 * (int64_t)atoms[j], x, prm[order[j] * n + qn], &inb)) return false;
        if (!inb) need_path = true;
    }
    if (!need_path) return true;
    double Bmin[3] = {-INFINITY, -INFINITY, -INFINITY};
    double Bmax[3] = {INFINITY, INFINITY, INFINITY};
    for (int j = 0; j <= lev; j++) {
        const double *cj = xyz + 3 * (int64_t)atoms[j];
        double bj = prm[order[j] * n + qn].b;
        for (int i = 0; i < 3; i++) {
            double lo = __dsub_rn(cj[i], bj), hi = __dadd_rn(cj[i], bj);
            Bmin[i] = Bmin[i] > lo ? Bmin[i] : lo;
            Bmax[i] = Bmax[i] < hi ? Bmax[i] : hi;
        }
    }
    return kd_path_reaches(leaf_atom_list, mc, cr, xyz, Bmin, Bmax);
}

// Search profile probes (PJG_SEARCH_PROF builds): lane 0 of each warp adds
// to its row of a shared array, flushed to sa.prof when the warp exits.
// The value argument is evaluated by lane 0 alone: it must not contain a
// warp-collective (ballot, shuffle), which every lane has to execute.
#if PJG_SEARCH_PROF
#define SPROF_ADD(i, v)                                                     \
    do {                                                                    \
        if (lane == 0) sprof[wib][i] += (unsigned long long)(v);            \
    } while (0)
#define SPROF_T(name) const long long name = clock64()
#define SPROF_CYC(i, t0) SPROF_ADD(i, clock64() - (t0))
// queue-empty and exit times of the warps of one k_search launch (ns)
__device__ unsigned long long g_search_tail[2];
#else
#define SPROF_ADD(i, v) \
    do {                \
    } while (0)
#define SPROF_T(name)
#define SPROF_CYC(i, t0) \
    do {                 \
    } while (0)
#endif

// CUT: the max_candidates cut applied inline (non-best mode with
// max_candidates); the other queries get a kernel without that code (its
// FP64 superposition in the loop costs registers everywhere).
template <typename PosT, bool FP32, bool CUT>
__global__ void __launch_bounds__(SEARCH_WARPS * 32, PJG_SEARCH_MIN_BLOCKS)
    k_search(ChunkView cv, TemplateView tv, CandView cd, SearchArgs sa, int32_t *pair_counter,
             const int32_t *scanned, CompleteRows out, unsigned long long *counters, LeafDemand dm) {
    extern __shared__ __align__(16) unsigned char smem[];
    using E = Entry<PosT>;
    const int lane = lane_id();
    const int wib = threadIdx.x >> 5;
#if PJG_SEARCH_PROF
    __shared__ unsigned long long sprof[SEARCH_WARPS][SP_NUM];
    if (lane < SP_NUM) sprof[wib][lane] = 0;
    __syncwarp();
    unsigned long long sp_fp64 = 0;  // this lane's FP64 decisions
#endif
    unsigned char *wbase = smem + (size_t)wib * sa.warp_smem;
    PairState &st = *reinterpret_cast<PairState *>(wbase);
    if (lane <= C_BYTES_EXP) st.acc[lane] = 0;
    __syncwarp();
    const size_t o2 = (sizeof(PairState) + 15) & ~size_t(15);
    E *tiles = reinterpret_cast<E *>(wbase + o2);
    const int64_t tile_units = (int64_t)(sa.warp_smem - o2) / (int64_t)sizeof(E);
    const int T = tv.n_templates;
    const int G = cd.n_sigs;
    // wall-time budget: every warp stops taking work, and stops the pair it
    // is on, once budget_ns have passed since it started (error code 3)
    uint64_t t_start = 0;
    if (lane == 0) t_start = global_ns();
    bool timed_out = false;
    uint32_t ticks = 0;
    auto over_budget = [&]() -> bool {
        if ((++ticks & 255u) != 0) return timed_out;
        int over = 0;
        if (lane == 0) over = (global_ns() - t_start) > sa.budget_ns;
        over = __shfl_sync(FULL_MASK, over, 0);
        if (over && !timed_out) {
            timed_out = true;
            if (lane == 0) atomicMax(&counters[C_ERROR], 3ull);
        }
        return timed_out;
    };

    // pairs of this round: every pair of the chunk, or the pairs that an
    // earlier round suspended (each with the rows it has already emitted)
    const bool fresh = dm.resume == nullptr;
    // a fresh round takes the heavy pairs first, then every pair in order
    // (skipping the heavy ones)
    const int n_heavy = fresh && dm.heavy ? (int)*dm.n_heavy : 0;
    const int n_items = fresh ? sa.n_pairs + n_heavy : dm.n_resume;
    // work queue: a warp takes sa.pair_grain consecutive items at a time
    int g_next = 0, g_end = 0;
    for (;;) {
        if (g_next >= g_end) {
            int base = 0;
            if (lane == 0) base = atomicAdd(pair_counter, sa.pair_grain);
            g_next = __shfl_sync(FULL_MASK, base, 0);
            g_end = g_next + sa.pair_grain;
        }
        const int item = g_next++;
        if (item >= n_items || timed_out) break;
        int pair;
        if (!fresh) {
            pair = dm.resume[item].pair;
        } else if (item < n_heavy) {
            pair = dm.heavy[item];
        } else {
            pair = item - n_heavy;
            if (n_heavy && dm.heavy_flag[pair]) continue;
        }
        SPROF_T(t_pair);
        SPROF_ADD(SP_PAIRS, 1);
        const int64_t skip = fresh ? 0 : dm.resume[item].skip;
        const int64_t saved = fresh ? -1 : dm.resume[item].state;
        const int s = pair / T;
        const int t = pair % T;
        const int ab = tv.atom_begin[t];
        const int n = tv.atom_begin[t + 1] - ab;
        // templates of more than 32 atoms are searched by k_search_large
        if (n <= 0 || n > 32) continue;
        const int64_t abase = cv.atom_base[s];
        const double *xyz64 = cv.xyz64 + 3 * abase;

        // ---- candidate-list lengths, empty-set skip, statistics
        int k = lane;
        int c = INT_MAX, sc = 0;
        if (k < n) {
            int64_t lw = (int64_t)s * G + tv.sig[ab + k];
            c = cd.count[lw];
            sc = scanned[lw];
        }
        unsigned zero = __ballot_sync(FULL_MASK, k < n && c == 0);
        int kstop = zero ? __ffs(zero) - 1 : n - 1;
        {
            int64_t bc = (k <= kstop && k < n) ? 8LL * sc + 16LL * c : 0;
            int64_t cc = (k <= kstop && k < n) ? (int64_t)c : 0;
            for (int o = 16; o; o >>= 1) {
                bc += __shfl_xor_sync(FULL_MASK, bc, o);
                cc += __shfl_xor_sync(FULL_MASK, cc, o);
            }
            if (lane == 0 && fresh) {
                st.acc[C_PAIRS] += 1ull;
                st.acc[C_BYTES_CAND] += (unsigned long long)bc;
                st.acc[C_CAND] += (unsigned long long)cc;
            }
        }
        if (zero) {
            SPROF_ADD(SP_EMPTY, 1);
            SPROF_CYC(SP_CYC_PAIR, t_pair);
            continue;
        }

        // ---- level order (stable by list length, ties by index)
        int rank = k;
        if (sa.reorder) {
            rank = 0;
            for (int j = 0; j < n; j++) {
                int cj = __shfl_sync(FULL_MASK, c, j);
                if (cj < c || (cj == c && j < k)) rank++;
            }
        }
        __syncwarp();
        if (k < n) st.order[rank] = k;
        __syncwarp();
        // tile capacity: equal entry count for levels 0..n-2
        int cap = n >= 2 ? (int)min((int64_t)sa.tile_cap, tile_units / (n - 1)) : 0;
        // levels whose list is in kd leaf order (level 0 reads the
        // candidate order)
        bool lvl_ready = true;
        if (lane < n) {
            int tk = st.order[lane];
            int64_t w2 = (int64_t)s * G + tv.sig[ab + tk];
            if (dm.state && lane > 0) lvl_ready = dm.state[w2] == 2;
            // level 0 reads the list in candidate order, the others in kd
            // leaf order (their leaf offset is set once the list is ordered)
            st.lvl_off[lane] = lane == 0 ? cd.offset[w2] : cd.leaf_offset[w2];
            st.blk_off[lane] = cd.blk_offset[w2];
            st.lvl_cnt[lane] = cd.count[w2];
            st.tkey[lane] = tv.key[ab + tk];
            st.F[lane] = 0;
            st.cnt[lane] = 0;
            st.par[lane] = 0;
            st.cnd[lane] = 0;
            st.tile[lane] = cap * lane;
        }
        const unsigned ready_mask = __ballot_sync(FULL_MASK, lvl_ready);
        bool suspended = false;
        __syncwarp();
        if (n >= 2 && cap < 32) {
            if (lane == 0) atomicMax(&counters[C_ERROR], 2ull);
            continue;
        }
        // annulus parameters of template atoms (p, q): prm[p * n + q]
        const AnnulusParam *prm = tv.params + tv.param_begin[t];

        int64_t emitted = 0;
        unsigned long long rechecks = 0;
        const int m0 = st.lvl_cnt[0];
        const int64_t off0 = st.lvl_off[0];

        // atom of level j at tile entry value pos: level-0 entries hold the
        // atom itself (the seeds' candidate-order positions are only a
        // cursor), deeper ones the position in the level's leaf order
        auto level_atom = [&](int j, int pos) -> int32_t {
            return j == 0 ? pos : cd.leaf_atom[st.lvl_off[j] + pos];
        };
        auto level_xyz = [&](int j, int pos) -> float4 {
            return j == 0 ? cv.xyz32[abase + pos] : cd.leaf_xyz[st.lvl_off[j] + pos];
        };

        bool stop = false;
        int64_t cut_base = 0;
        const int64_t stop_at = (sa.best_match && sa.max_candidates >= 0) ? (int64_t)sa.max_candidates + 2 : -1;

        // emit complete rows: lanes with `pass`, level positions in pos[]
        // (levels 0..n-2) and the last level's position `lastpos`
        auto emit = [&](bool pass, const int32_t *pos, int lastpos) -> void {
            unsigned m = __ballot_sync(FULL_MASK, pass);
            if (!m) return;
            SPROF_T(t_emit);
            double rm = 0.0;
            int32_t at[32];
            if (pass) {
                for (int j = 0; j < n - 1; j++) at[st.order[j]] = level_atom(j, pos[j]);
                at[st.order[n - 1]] = level_atom(n - 1, lastpos);
            }
            if (CUT) {
                // Query.__next__'s max_candidates cut, applied while
                // searching: the candidate whose distance from the last hit
                // (or the template start) reaches M+1 ends the template's
                // stream after it has been considered
                bool hitf = false;
                if (pass) {
                    rm = lane_rmsd(n, at, xyz64, tv.pos + 3 * (int64_t)ab);
                    hitf = rm <= sa.rmsd_threshold && n >= 3;
                }
                unsigned hl = __ballot_sync(FULL_MASK, hitf);
                unsigned mm = m;
                int r = 0, keep = 32;
                while (mm) {
                    int ln = __ffs(mm) - 1;
                    mm &= mm - 1;
                    int64_t q = emitted + r;
                    if (q - cut_base == (int64_t)sa.max_candidates + 1) {
                        keep = r;
                        stop = true;
                        break;
                    }
                    if ((hl >> ln) & 1u) cut_base = q + 1;
                    r++;
                }
                int myrank = __popc(m & ((1u << lane) - 1u));
                pass = pass && myrank <= keep;
                m = __ballot_sync(FULL_MASK, pass);
            }
            int np = __popc(m);
            // rows before `skip` were emitted before the pair was suspended
            const int64_t seen = skip - emitted;
            const int nold = seen <= 0 ? 0 : seen >= np ? np : (int)seen;
            int64_t base = 0;
            if (lane == 0 && np > nold) base = (int64_t)atomicAdd(out.count, (unsigned long long)(np - nold));
            base = __shfl_sync(FULL_MASK, base, 0);
            if (pass && __popc(m & ((1u << lane) - 1u)) >= nold) {
                int rk = __popc(m & ((1u << lane) - 1u));
                int64_t ri = base + rk - nold;
                if (ri < out.capacity) {
                    int32_t *dst = out.atoms + ri * out.stride;
                    for (int j = 0; j < n; j++) dst[j] = at[j];
                    out.pair[ri] = pair;
                    out.ordinal[ri] = emitted + rk;
                    if (out.rmsd) out.rmsd[ri] = rm;
                }
            }
            emitted += np;
            if (stop_at >= 0 && emitted >= stop_at) stop = true;
            SPROF_ADD(SP_ROWS, np);
            SPROF_CYC(SP_CYC_EMIT, t_emit);
        };

        SPROF_CYC(SP_CYC_SETUP, t_pair);
        if (n == 1) {
            // Scanner_next with one level advances the seed index before
            // reporting (patches/Scanner.c.patch:244-263): seeds 1..m0-1
            for (int b = 1; b < m0 && !stop; b += 32) {
                int p = b + lane;
                emit(p < m0, nullptr, p < m0 ? cd.cand_atom[off0 + p] : 0);
                if (over_budget()) stop = true;
            }
            if (lane == 0) st.F[0] = m0;
        } else {
            int root = 0;
            int lev = -1;
            int chain_lev = -1, chain_par = -1;
            float box_lo[3], box_hi[3];
            if (saved >= 0) {
                // resume a suspended pair from its saved state
                const unsigned char *b = dm.pool_in + saved;
                const SavedPair h = *reinterpret_cast<const SavedPair *>(b);
                root = h.root;
                lev = h.lev;
                emitted = h.emitted;
                cut_base = h.cut_base;
                if (lane == 0) rechecks = h.rechecks;
                const int64_t hdr = (int64_t)sizeof(SavedPair) + 16LL * (lev + 1);
                int4 c4 = make_int4(0, 0, 0, 0);
                if (lane <= lev) {
                    c4 = reinterpret_cast<const int4 *>(b + sizeof(SavedPair))[lane];
                    st.F[lane] = c4.x;
                    st.cnt[lane] = c4.y;
                    st.par[lane] = c4.z;
                    st.cnd[lane] = c4.w;
                }
                int tile_pre = c4.y;
                for (int o = 1; o < 32; o <<= 1) {
                    int v = __shfl_up_sync(FULL_MASK, tile_pre, o);
                    if (lane >= o) tile_pre += v;
                }
                const E *srcb = reinterpret_cast<const E *>(b + hdr);
                for (int j = 0; j <= lev; j++) {
                    const int cj = __shfl_sync(FULL_MASK, c4.y, j);
                    const int pj = __shfl_sync(FULL_MASK, tile_pre, j) - cj;
                    E *dst = tiles + st.tile[j];
                    for (int i = lane; i < cj; i += 32) dst[i] = srcb[pj + i];
                }
                __syncwarp();
            }
            while (!stop) {
                if (over_budget()) break;
                SPROF_ADD(SP_LOOP_ITERS, 1);
                SPROF_T(t_it);
                if (lev < 0) {
                    if (root >= m0) break;
                    SPROF_T(t_seed);
                    int kk = min(cap, m0 - root);
                    E *t0 = tiles + st.tile[0];
                    for (int i = lane; i < kk; i += 32) {
                        E e;
                        e.pos = (PosT)cd.cand_atom[off0 + root + i];
                        e.parent = 0;
                        t0[i] = e;
                    }
                    root += kk;
                    __syncwarp();
                    if (lane == 0) {
                        st.F[0] += kk;
                        st.cnt[0] = kk;
                        st.par[0] = 0;
                        st.cnd[0] = 0;
                    }
                    __syncwarp();
                    lev = 0;
                    chain_lev = -1;
                    SPROF_CYC(SP_CYC_SEED, t_seed);
                    continue;
                }
                const int child = lev + 1;
                const bool last = (child == n - 1);
                const int pcnt = st.cnt[lev];
                const int ppar = st.par[lev];
                const int ccnt = last ? 0 : st.cnt[child];
                if (ppar >= pcnt) {
                    __syncwarp();
                    if (!last && ccnt > 0) {
                        if (lane == 0) {
                            st.par[child] = 0;
                            st.cnd[child] = 0;
                        }
                        __syncwarp();
                        lev = child;
                        SPROF_CYC(SP_CYC_CTRL, t_it);
                        continue;
                    }
                    if (lane == 0) st.cnt[lev] = 0;
                    __syncwarp();
                    lev--;
                    SPROF_CYC(SP_CYC_CTRL, t_it);
                    continue;
                }
                if (!((ready_mask >> child) & 1u)) {
                    // the child level's list has no kd leaf order yet:
                    // request it and suspend the pair until the next round.
                    // Its child tile and every deeper one are empty here, so
                    // the state is the header, the cursors of levels 0..lev
                    // and the used entries of their tiles.
                    unsigned long long rs = rechecks;
                    for (int o = 16; o; o >>= 1) rs += __shfl_xor_sync(FULL_MASK, rs, o);
                    int used = lane <= lev ? st.cnt[lane] : 0;
                    int tile_pre = used;  // inclusive prefix over levels
                    for (int o = 1; o < 32; o <<= 1) {
                        int v = __shfl_up_sync(FULL_MASK, tile_pre, o);
                        if (lane >= o) tile_pre += v;
                    }
                    const int total = __shfl_sync(FULL_MASK, tile_pre, 31);
                    const int64_t hdr = (int64_t)sizeof(SavedPair) + 16LL * (lev + 1);
                    const int64_t bytes = (hdr + (int64_t)total * (int64_t)sizeof(E) + 15) & ~15LL;
                    int64_t off = -1;
                    if (lane == 0 && dm.pool_out) {
                        unsigned long long o = atomicAdd(dm.pool_used, (unsigned long long)bytes);
                        if ((int64_t)o + bytes <= dm.pool_cap) off = (int64_t)o;
                    }
                    off = __shfl_sync(FULL_MASK, off, 0);
                    if (off >= 0) {
                        unsigned char *b = dm.pool_out + off;
                        if (lane == 0) {
                            SavedPair h;
                            h.root = root;
                            h.lev = lev;
                            h.emitted = emitted;
                            h.cut_base = cut_base;
                            h.rechecks = rs;
                            *reinterpret_cast<SavedPair *>(b) = h;
                        }
                        if (lane <= lev)
                            reinterpret_cast<int4 *>(b + sizeof(SavedPair))[lane] =
                                make_int4(st.F[lane], st.cnt[lane], st.par[lane], st.cnd[lane]);
                        E *dst = reinterpret_cast<E *>(b + hdr);
                        for (int j = 0; j <= lev; j++) {
                            const int cj = __shfl_sync(FULL_MASK, used, j);
                            const int pj = __shfl_sync(FULL_MASK, tile_pre, j) - cj;
                            const E *src = tiles + st.tile[j];
                            for (int i = lane; i < cj; i += 32) dst[pj + i] = src[i];
                        }
                    }
                    // request the list of this level and of the next
                    // sa.leaf_reach - 1 deeper ones, or of every deeper
                    // one (leaf_reach < 0: a resumed pair then never stops
                    // again, a chunk takes at most two search rounds)
                    if (lane >= child && lane < n && (sa.leaf_reach < 0 || lane < child + sa.leaf_reach) &&
                        !((ready_mask >> lane) & 1u))
                        request_list(dm, (int64_t)s * G + tv.sig[ab + st.order[lane]], st.lvl_cnt[lane]);
                    if (lane == 0) {
                        Suspended sp;
                        sp.pair = pair;
                        sp.pad = 0;
                        sp.skip = off >= 0 ? 0 : (emitted > skip ? emitted : skip);
                        sp.state = off;
                        dm.suspended[atomicAdd(dm.n_suspended, 1ull)] = sp;
                    }
                    suspended = true;
                    SPROF_CYC(SP_CYC_SUSP, t_it);
                    break;
                }
                const int mc = st.lvl_cnt[child];
                const int qn = st.order[child];
                const int32_t tn = st.tkey[child];
                const int64_t coff = st.lvl_off[child];
                const E *ptile = tiles + st.tile[lev];
                E *ctile = tiles + st.tile[child];
                bool pass = false;
                int cr = 0;
                int my_parent = 0;      // product mode: this lane's parent entry
                int32_t chainpos[32];   // product mode: this lane's parent chain
                SPROF_CYC(SP_CYC_CTRL, t_it);
                SPROF_T(t_exp);
                if (mc >= sa.block_min) {
                    // ---------------- block mode ----------------
                    if (!last && cap - ccnt < 32) {
                        __syncwarp();
                        if (lane == 0) {
                            st.par[child] = 0;
                            st.cnd[child] = 0;
                        }
                        __syncwarp();
                        lev = child;
                        continue;
                    }
                    // The parent's chain, then every block from the cursor on
                    // whose bounding box meets the join box, in leaf order.
                    // Each lane tests its leaf against the join box; the
                    // leaves inside it go to a queue in shared memory, and the
                    // full test (chain/residue rules, FP32 annuli, FP64
                    // recheck) runs on batches of 32 queued leaves, so the
                    // children (or complete rows) come out in leaf order.  The
                    // cursor st.cnd[lev] is the first leaf position not yet
                    // tested; the parent is left early only when the child
                    // tile cannot take another batch.  The boxes of the first
                    // 32 blocks do not depend on the chain: their loads are
                    // issued before the chain is gathered.
                    SPROF_ADD(SP_BLOCK_VISITS, 1);
                    SPROF_ADD(SP_BLOCK_VISITS_L0, lev == 0);
                    const int nblk = (mc + CULL_BLK - 1) / CULL_BLK;
                    const int pstart = st.cnd[lev];
                    const int gfirst = pstart / CULL_BLK;
                    const int64_t boff = st.blk_off[child];
                    float4 bl = make_float4(0.f, 0.f, 0.f, 0.f), bh = bl;
                    if (gfirst + lane < nblk) {
                        bl = cd.blk_lo[boff + gfirst + lane];
                        bh = cd.blk_hi[boff + gfirst + lane];
                    }
                    SPROF_T(t_chain);
                    if (chain_lev != lev || chain_par != ppar) {
                        const E pe = tiles[st.tile[lev] + ppar];
                        float olo[3] = {-INFINITY, -INFINITY, -INFINITY}, ohi[3] = {INFINITY, INFINITY, INFINITY};
                        if (chain_lev == lev && (int)pe.parent == st.chain_gp) {
                            // a sibling of the previous parent (every seed is
                            // one of the previous seed): levels below lev are
                            // unchanged, only this parent's point and box are
                            // new
                            SPROF_ADD(SP_CHAIN_SIBLING, 1);
                            if (lane == lev) {
                                const float4 cj = level_xyz(lev, (int)pe.pos);
                                st.cxyz[lev] = cj;
                                st.cpos[lev] = (int)pe.pos;
                                const float rb = sqrtf(fmaxf(st.cthr[lev].w, 0.f)) * 1.000001f + 1e-3f;
                                olo[0] = cj.x - rb;
                                olo[1] = cj.y - rb;
                                olo[2] = cj.z - rb;
                                ohi[0] = cj.x + rb;
                                ohi[1] = cj.y + rb;
                                ohi[2] = cj.z + rb;
                            }
                        } else {
                            // positions of the parent's chain, by walking the tiles
                            SPROF_ADD(SP_CHAIN_FULL, 1);
                            __syncwarp();
                            if (lane == 0) {
                                int idx = ppar;
                                for (int j = lev; j >= 0; j--) {
                                    E e = tiles[st.tile[j] + idx];
                                    st.cpos[j] = (int)e.pos;
                                    idx = e.parent;
                                }
                                st.chain_gp = (int)pe.parent;
                            }
                            __syncwarp();
                            float lo[3] = {-INFINITY, -INFINITY, -INFINITY}, hi[3] = {INFINITY, INFINITY, INFINITY};
                            if (lane <= lev) {
                                float4 cj = level_xyz(lane, st.cpos[lane]);
                                float4 th = prm[st.order[lane] * n + qn].thr;
                                st.cxyz[lane] = cj;
                                st.cthr[lane] = th;
                                float rb = sqrtf(fmaxf(th.w, 0.f)) * 1.000001f + 1e-3f;
                                lo[0] = cj.x - rb;
                                lo[1] = cj.y - rb;
                                lo[2] = cj.z - rb;
                                hi[0] = cj.x + rb;
                                hi[1] = cj.y + rb;
                                hi[2] = cj.z + rb;
                            }
                            if (lane == lev)
                                for (int i = 0; i < 3; i++) {
                                    olo[i] = lo[i];
                                    ohi[i] = hi[i];
                                }
                            // join box of levels below lev (kept for siblings)
                            for (int i = 0; i < 3; i++) {
                                float a = lane < lev ? lo[i] : -INFINITY, b = lane < lev ? hi[i] : INFINITY;
                                for (int off = 16; off; off >>= 1) {
                                    a = fmaxf(a, __shfl_xor_sync(FULL_MASK, a, off));
                                    b = fminf(b, __shfl_xor_sync(FULL_MASK, b, off));
                                }
                                if (lane == 0) {
                                    st.pbox[i] = a;
                                    st.pbox[3 + i] = b;
                                }
                            }
                            __syncwarp();
                        }
                        // the parent's own box, from lane lev, met with the
                        // prefix box
                        for (int i = 0; i < 3; i++) {
                            box_lo[i] = fmaxf(st.pbox[i], __shfl_sync(FULL_MASK, olo[i], lev));
                            box_hi[i] = fminf(st.pbox[3 + i], __shfl_sync(FULL_MASK, ohi[i], lev));
                        }
                        __syncwarp();
                        chain_lev = lev;
                        chain_par = ppar;
                        __syncwarp();
                    }
                    SPROF_CYC(SP_CYC_CHAIN, t_chain);
                    int ncnt = ccnt;
                    int resume = -1;
                    int queued = 0;
                    // the parent's point and its annulus bounds to the child
                    const float4 pxyz = st.cxyz[lev];
                    const float4 pthr = st.cthr[lev];
                    // full test of queue entries 0..k-1 (lane i takes entry i),
                    // then the entries after them move to the queue's front
                    auto run_batch = [&](int k) {
                        SPROF_T(t_batch);
                        SPROF_ADD(SP_BATCHES, 1);
                        SPROF_ADD(SP_BATCH_LANES, k);
                        cr = lane < k ? st.qpos[lane] : 0;
                        const float4 xc = lane < k ? st.qxyz[lane] : make_float4(0.f, 0.f, 0.f, 0.f);
                        pass = false;
                        if (lane < k) {
                            const int32_t kn = __float_as_int(xc.w);
                            pass = true;
                            unsigned exact = 0;
                            for (int j = 0; j <= lev; j++) {
                                const float4 xj = st.cxyz[j];
                                if (!check_pair(__float_as_int(xj.w), kn, st.tkey[j], tn, sa.ignore_chain)) {
                                    pass = false;
                                    break;
                                }
                                if (FP32) {
                                    const float dx = xj.x - xc.x, dy = xj.y - xc.y, dz = xj.z - xc.z;
                                    const float d2 = dx * dx + dy * dy + dz * dz;
                                    const float4 th = st.cthr[j];
                                    if (d2 < th.x || d2 > th.w) {
                                        pass = false;
                                        break;
                                    }
                                    if (!(d2 >= th.y && d2 <= th.z)) exact |= 1u << j;
                                } else {
                                    exact |= 1u << j;
                                }
                            }
                            if (pass && exact) {
                                if (FP32) rechecks += __popc(exact);
#if PJG_SEARCH_PROF
                                sp_fp64++;
#endif
                                int32_t atoms[32];
                                for (int j = 0; j <= lev; j++) atoms[j] = level_atom(j, st.cpos[j]);
                                pass = decide_fp64(exact, lev, atoms, cd.leaf_atom[coff + cr], xyz64, prm, st.order,
                                                   n, qn, cd.leaf_atom + coff, mc, cr);
                            }
                        }
                        const unsigned m = __ballot_sync(FULL_MASK, pass);
                        SPROF_ADD(SP_CHILD_BLOCK, __popc(m));
                        if (last) {
                            emit(pass, st.cpos, cr);
                        } else if (pass) {
                            E e;
                            e.pos = (PosT)cr;
                            e.parent = (uint16_t)ppar;
                            ctile[ncnt + __popc(m & ((1u << lane) - 1u))] = e;
                        }
                        if (!last) ncnt += __popc(m);
                        if (lane == 0) st.F[child] += __popc(m);
                        const int rest = queued - k;
                        int qp = 0;
                        float4 qx = make_float4(0.f, 0.f, 0.f, 0.f);
                        __syncwarp();
                        if (lane < rest) {
                            qp = st.qpos[k + lane];
                            qx = st.qxyz[k + lane];
                        }
                        __syncwarp();
                        if (lane < rest) {
                            st.qpos[lane] = qp;
                            st.qxyz[lane] = qx;
                        }
                        __syncwarp();
                        queued = rest;
                        SPROF_CYC(SP_CYC_BATCH, t_batch);
                    };
                    for (int g0 = gfirst; g0 < nblk && resume < 0 && !stop; g0 += 32) {
                        const int b = g0 + lane;
                        bool hit = false;
                        if (b < nblk) {
                            hit = !(bl.x > box_hi[0] || bh.x < box_lo[0] || bl.y > box_hi[1] || bh.y < box_lo[1] ||
                                    bl.z > box_hi[2] || bh.z < box_lo[2]);
                        }
                        // boxes of the next 32 blocks, loaded while these are
                        // processed
                        if (b + 32 < nblk) {
                            bl = cd.blk_lo[boff + b + 32];
                            bh = cd.blk_hi[boff + b + 32];
                        }
                        unsigned hm = __ballot_sync(FULL_MASK, hit);
                        SPROF_ADD(SP_G0_ITERS, 1);
                        SPROF_ADD(SP_BLOCKS_TESTED, min(32, nblk - g0));
                        SPROF_ADD(SP_BLOCKS_HIT, __popc(hm));
                        // hit blocks in order, 32 / CULL_BLK of them a step:
                        // lane l takes leaf l % CULL_BLK of the step's
                        // (l / CULL_BLK)-th hit block; the leaves of the next
                        // step are loaded while the current one is queued
                        constexpr int GRP = 32 / CULL_BLK;
                        const int slot = lane / CULL_BLK;
                        auto step_leaf = [&](unsigned &h) -> int {
                            // this lane's leaf position in the next step (-1:
                            // its slot has no block), the step's blocks
                            // removed from h
                            unsigned hh = h;
                            for (int i = 0; i < slot; i++) hh &= hh - 1;
                            const int q = hh ? (g0 + __ffs(hh) - 1) * CULL_BLK + (lane & (CULL_BLK - 1)) : -1;
                            for (int i = 0; i < GRP; i++) h &= h - 1;
                            return q;
                        };
                        bool have = hm != 0;
                        int qnext = -1;
                        float4 xn = make_float4(0.f, 0.f, 0.f, 0.f);
                        if (have) {
                            qnext = step_leaf(hm);
                            if (qnext >= 0 && qnext < mc) xn = cd.leaf_xyz[coff + qnext];
                        }
                        while (have) {
                            const int q = qnext;
                            const float4 xc = xn;
                            have = hm != 0;
                            if (have) {
                                qnext = step_leaf(hm);
                                if (qnext >= 0 && qnext < mc) xn = cd.leaf_xyz[coff + qnext];
                            }
                            // inside the join box and not certainly outside
                            // the parent's own annulus (the FP32 reject
                            // bounds of the full test, so the full test
                            // would reject the same leaves)
                            bool inb = q >= 0 && q < mc && q >= pstart &&
                                       !(xc.x < box_lo[0] || xc.x > box_hi[0] || xc.y < box_lo[1] ||
                                         xc.y > box_hi[1] || xc.z < box_lo[2] || xc.z > box_hi[2]);
                            if (FP32 && inb) {
                                const float dx = pxyz.x - xc.x, dy = pxyz.y - xc.y, dz = pxyz.z - xc.z;
                                const float d2 = dx * dx + dy * dy + dz * dz;
                                inb = !(d2 < pthr.x || d2 > pthr.w);
                            }
                            const unsigned im = __ballot_sync(FULL_MASK, inb);
                            SPROF_ADD(SP_LEAVES_INBOX, __popc(im));
                            if (inb) {
                                const int qi = queued + __popc(im & ((1u << lane) - 1u));
                                st.qpos[qi] = q;
                                st.qxyz[qi] = xc;
                            }
                            queued += __popc(im);
                            __syncwarp();
                            if (queued >= 32) {
                                if (!last && cap - ncnt < 32) {
                                    // child tile full: finish it first, then
                                    // come back to this parent at the queue's
                                    // first leaf
                                    resume = st.qpos[0];
                                    break;
                                }
                                run_batch(32);
                                if (stop) break;
                            }
                        }
                        if (over_budget()) stop = true;
                    }
                    if (resume < 0 && !stop && queued > 0) {
                        if (!last && cap - ncnt < 32) resume = st.qpos[0];
                        else run_batch(queued);
                    }
                    __syncwarp();
                    if (lane == 0) {
                        if (!last) st.cnt[child] = ncnt;
                        if (resume >= 0) {
                            st.cnd[lev] = resume;
                            st.par[child] = 0;
                            st.cnd[child] = 0;
                        } else {
                            st.par[lev] = ppar + 1;
                            st.cnd[lev] = 0;
                        }
                    }
                    __syncwarp();
                    if (resume >= 0) lev = child;
                    SPROF_CYC(SP_CYC_BLOCK, t_exp);
                    continue;
                } else {
                    // ---------------- product mode ----------------
                    int batch = last ? 32 : min(32, cap - ccnt);
                    if (batch <= 0) {
                        __syncwarp();
                        if (lane == 0) {
                            st.par[child] = 0;
                            st.cnd[child] = 0;
                        }
                        __syncwarp();
                        lev = child;
                        continue;
                    }
                    const int pcnd = st.cnd[lev];
                    const int tt = pcnd + lane;
                    // (parent, candidate) of product position tt: divmod by
                    // mc through a float reciprocal, corrected to exact
                    const float rmc = __frcp_rn((float)mc);
                    auto divmod = [&](int x, int &q, int &r) {
                        q = __float2int_rz(__int2float_rn(x) * rmc);
                        r = x - q * mc;
                        if (r < 0) {
                            q--;
                            r += mc;
                        } else if (r >= mc) {
                            q++;
                            r -= mc;
                        }
                    };
                    int pq;
                    divmod(tt, pq, cr);
                    const int p = ppar + pq;
                    const bool valid = lane < batch && p < pcnt;
                    SPROF_ADD(SP_PROD_BATCHES, 1);
                    SPROF_ADD(SP_PROD_BATCHES_L0, lev == 0);
#if PJG_SEARCH_PROF
                    {
                        // every lane takes part in the ballot; lane 0 adds
                        const unsigned vm = __ballot_sync(FULL_MASK, valid);
                        SPROF_ADD(SP_PROD_LANES, __popc(vm));
                    }
#endif
                    if (valid) {
                        // the parent chain walked up from the parent, each
                        // level tested as it is reached (the first failing
                        // test ends the walk)
                        const float4 xc = cd.leaf_xyz[coff + cr];
                        const int32_t kn = __float_as_int(xc.w);
                        pass = true;
                        unsigned exact = 0;
                        int idx = p;
                        for (int j = lev; j >= 0; j--) {
                            const E e = tiles[st.tile[j] + idx];
                            idx = e.parent;
                            const float4 xj = level_xyz(j, (int)e.pos);
                            if (!check_pair(__float_as_int(xj.w), kn, st.tkey[j], tn, sa.ignore_chain)) {
                                pass = false;
                                break;
                            }
                            if (FP32) {
                                float dx = xj.x - xc.x, dy = xj.y - xc.y, dz = xj.z - xc.z;
                                float d2 = dx * dx + dy * dy + dz * dz;
                                float4 th = prm[st.order[j] * n + qn].thr;
                                if (d2 < th.x || d2 > th.w) {
                                    pass = false;
                                    break;
                                }
                                if (!(d2 >= th.y && d2 <= th.z)) exact |= 1u << j;
                            } else {
                                exact |= 1u << j;
                            }
                        }
                        if (pass && (last || exact)) {
                            // positions of the chain (passing lanes): the
                            // row's atoms, the FP64 recheck
                            int ix = p;
                            for (int j = lev; j >= 0; j--) {
                                const E e = tiles[st.tile[j] + ix];
                                chainpos[j] = (int)e.pos;
                                ix = e.parent;
                            }
                        }
                        if (pass && exact) {
                            if (FP32) rechecks += __popc(exact);
#if PJG_SEARCH_PROF
                            sp_fp64++;
#endif
                            int32_t atoms[32];
                            for (int j = 0; j <= lev; j++) atoms[j] = level_atom(j, chainpos[j]);
                            pass = decide_fp64(exact, lev, atoms, cd.leaf_atom[coff + cr], xyz64, prm, st.order, n,
                                               qn, cd.leaf_atom + coff, mc, cr);
                        }
                    }
                    // advance the parent cursor by `batch` product positions
                    int np2, nc2;
                    divmod(pcnd + batch, np2, nc2);
                    np2 += ppar;
                    if (np2 >= pcnt) {
                        np2 = pcnt;
                        nc2 = 0;
                    }
                    __syncwarp();
                    if (lane == 0) {
                        st.par[lev] = np2;
                        st.cnd[lev] = nc2;
                    }
                    __syncwarp();
                    my_parent = p;
                }
                // ---- children / complete rows
                const bool block_mode = mc >= sa.block_min;
                unsigned m = __ballot_sync(FULL_MASK, pass);
                SPROF_ADD(SP_CHILD_PROD, __popc(m));
                if (last) {
                    if (block_mode) {
                        emit(pass, st.cpos, cr);
                    } else {
                        emit(pass, chainpos, cr);
                    }
                    __syncwarp();
                    if (lane == 0) st.F[child] += __popc(m);
                    __syncwarp();
                    if (!block_mode) chain_lev = -1;
                } else {
                    if (pass) {
                        int ci = ccnt + __popc(m & ((1u << lane) - 1u));
                        E e;
                        e.pos = (PosT)cr;
                        e.parent = (uint16_t)(block_mode ? ppar : my_parent);
                        ctile[ci] = e;
                    }
                    int ncnt = ccnt + __popc(m);
                    __syncwarp();
                    if (lane == 0) {
                        st.cnt[child] = ncnt;
                        st.F[child] += __popc(m);
                    }
                    __syncwarp();
                    if (!block_mode) {
                        chain_lev = -1;
                        bool parent_done = st.par[lev] >= pcnt;
                        if (ncnt > 0 && (cap - ncnt < 32 || parent_done)) {
                            if (lane == 0) {
                                st.par[child] = 0;
                                st.cnd[child] = 0;
                            }
                            __syncwarp();
                            lev = child;
                        }
                    } else if (cap - ncnt < 32) {
                        if (lane == 0) {
                            st.par[child] = 0;
                            st.cnd[child] = 0;
                        }
                        __syncwarp();
                        lev = child;
                    }
                }
                SPROF_CYC(SP_CYC_PROD, t_exp);
            }
        }
        __syncwarp();
        SPROF_CYC(SP_CYC_PAIR, t_pair);
#if PJG_SEARCH_PROF
        if (lane == 0) {
            const unsigned long long c = (unsigned long long)(clock64() - t_pair);
            if (c > sprof[wib][SP_PAIR_MAX_CYC]) sprof[wib][SP_PAIR_MAX_CYC] = c;
        }
#endif
        if (suspended) continue;
        if (lane == 0 && emitted > 0) out.pair_rows[pair] = (int32_t)emitted;
        // ---- statistics of the pair
        for (int o = 16; o; o >>= 1) rechecks += __shfl_xor_sync(FULL_MASK, rechecks, o);
        if (lane == 0) {
            int64_t partials = 0, bexp = 0;
            for (int l = 0; l < n; l++) partials += st.F[l];
            for (int l = 1; l < n; l++)
                bexp += 4LL * l * st.F[l - 1] + (4LL * (l + 1) + 16) * st.F[l];
            st.acc[C_PARTIALS] += (unsigned long long)partials;
            st.acc[C_COMPLETE] += (unsigned long long)st.F[n - 1];
            st.acc[C_BYTES_EXP] += (unsigned long long)bexp;
            st.acc[C_RECHECK] += rechecks;
        }
        __syncwarp();
    }
#if PJG_SEARCH_PROF
    if (lane == 0) atomicMin(&g_search_tail[0], (unsigned long long)global_ns());
#endif
    __syncwarp();
    if (lane <= C_BYTES_EXP && st.acc[lane]) atomicAdd(&counters[lane], st.acc[lane]);
#if PJG_SEARCH_PROF
    for (int o = 16; o; o >>= 1) sp_fp64 += __shfl_xor_sync(FULL_MASK, sp_fp64, o);
    SPROF_ADD(SP_FP64, sp_fp64);
    __syncwarp();
    if (sa.prof && lane < SP_NUM) {
        if (lane == SP_PAIR_MAX_CYC) atomicMax(&sa.prof[lane], sprof[wib][lane]);
        else if (lane != SP_TAIL_NS) atomicAdd(&sa.prof[lane], sprof[wib][lane]);
    }
    if (lane == 0) atomicMax(&g_search_tail[1], (unsigned long long)global_ns());
#endif
}


// ---------------------------------------------------------------------------
// Search for templates of more than 32 atoms (k_search keeps one level per
// lane, so it takes at most 32).  Warp per pair, the reference's
// depth-first backtracking taken literally: one chain of atoms, and at each
// level the next 32 leaf positions tested by the lanes at once, the passing
// ones expanded one after the other in leaf order (their ballot mask is kept
// per level, so every position is tested once per parent).  Every distance
// test is the reference's FP64 arithmetic (annulus64, plus the kd path
// check for a point outside an annulus box).  Every list of these pairs is
// in kd leaf order before the first search round (k_demand_levels requests
// them all), so they never suspend.  Per-warp state in dynamic shared
// memory, 52 bytes a template atom (large_warp_bytes).

__device__ __forceinline__ bool decide_fp64_chain(int levp, const int32_t *catom, int32_t an, const double *xyz,
                                                  const AnnulusParam *prm, const int32_t *order, int n, int qn,
                                                  const int32_t *leaf_atom_list, int mc, int cr) {
    bool need_path = false;
    const double *x = xyz + 3 * (int64_t)an;
    for (int j = 0; j <= levp; j++) {
        bool inb;
        if (!annulus64(xyz + 3 * (int64_t)catom[j], x, prm[order[j] * n + qn], &inb)) return false;
        if (!inb) need_path = true;
    }
    if (!need_path) return true;
    double Bmin[3] = {-INFINITY, -INFINITY, -INFINITY};
    double Bmax[3] = {INFINITY, INFINITY, INFINITY};
    for (int j = 0; j <= levp; j++) {
        const double *cj = xyz + 3 * (int64_t)catom[j];
        const double bj = prm[order[j] * n + qn].b;
        for (int i = 0; i < 3; i++) {
            const double lo = __dsub_rn(cj[i], bj), hi = __dadd_rn(cj[i], bj);
            Bmin[i] = Bmin[i] > lo ? Bmin[i] : lo;
            Bmax[i] = Bmax[i] < hi ? Bmax[i] : hi;
        }
    }
    return kd_path_reaches(leaf_atom_list, mc, cr, xyz, Bmin, Bmax);
}

__global__ void __launch_bounds__(LARGE_WARPS * 32)
    k_search_large(ChunkView cv, TemplateView tv, CandView cd, SearchArgs sa, const int32_t *large, int32_t n_large,
                   int32_t *item_counter, const int32_t *scanned, CompleteRows out, unsigned long long *counters,
                   const int32_t *lstate) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = lane_id();
    const int nmax = tv.max_atoms;
    unsigned char *wb = smem + (size_t)(threadIdx.x >> 5) * large_warp_bytes(nmax);
    int64_t *lvl_off = reinterpret_cast<int64_t *>(wb);  // list offset of each level
    int64_t *F = lvl_off + nmax;                         // partial assignments per level
    int32_t *lvl_cnt = reinterpret_cast<int32_t *>(F + nmax);
    int32_t *order = lvl_cnt + nmax;                     // template atom of each level
    int32_t *tkey = order + nmax;                        // its key bits
    int32_t *catom = tkey + nmax;                        // chain: atom of each level
    int32_t *ckey = catom + nmax;                        //   its key bits
    int32_t *trow = ckey + nmax;                         //   atoms by template atom
    int32_t *next = trow + nmax;                         // next untested position per level
    int32_t *cbase = next + nmax;                        // first position of the last tested batch
    uint32_t *rem = reinterpret_cast<uint32_t *>(cbase + nmax);  // its passing lanes not yet expanded
    const int T = tv.n_templates, G = cd.n_sigs;
    uint64_t t_start = 0;
    if (lane == 0) t_start = global_ns();
    bool timed_out = false;
    uint32_t ticks = 0;
    const int64_t n_items = (int64_t)cv.n_structures * n_large;
    for (;;) {
        int64_t item = 0;
        if (lane == 0) item = atomicAdd(item_counter, 1);
        item = __shfl_sync(FULL_MASK, item, 0);
        if (item >= n_items || timed_out) break;
        const int s = (int)(item / n_large);
        const int t = large[item % n_large];
        const int pair = s * T + t;
        const int ab = tv.atom_begin[t];
        const int n = tv.atom_begin[t + 1] - ab;
        const int64_t abase = cv.atom_base[s];
        const double *xyz64 = cv.xyz64 + 3 * abase;
        // lengths, empty-set skip and statistics (template atom order), as
        // k_search
        int first_zero = n;
        for (int k = lane; k < n; k += 32) {
            const int c = cd.count[(int64_t)s * G + tv.sig[ab + k]];
            next[k] = c;  // lengths by template atom, for the level order
            if (c == 0) first_zero = min(first_zero, k);
        }
        for (int o = 16; o; o >>= 1) first_zero = min(first_zero, __shfl_xor_sync(FULL_MASK, first_zero, o));
        {
            const int kstop = first_zero < n ? first_zero : n - 1;
            long long bc = 0, cc = 0;
            for (int k = lane; k <= kstop; k += 32) {
                const int64_t lw = (int64_t)s * G + tv.sig[ab + k];
                bc += 8LL * scanned[lw] + 16LL * cd.count[lw];
                cc += cd.count[lw];
            }
            for (int o = 16; o; o >>= 1) {
                bc += __shfl_xor_sync(FULL_MASK, bc, o);
                cc += __shfl_xor_sync(FULL_MASK, cc, o);
            }
            if (lane == 0) {
                atomicAdd(&counters[C_PAIRS], 1ull);
                atomicAdd(&counters[C_BYTES_CAND], (unsigned long long)bc);
                atomicAdd(&counters[C_CAND], (unsigned long long)cc);
            }
        }
        __syncwarp();
        if (first_zero < n) continue;
        // level order: stable by list length, ties by index
        for (int k = lane; k < n; k += 32) {
            int r = k;
            if (sa.reorder) {
                const int ck = next[k];
                r = 0;
                for (int j = 0; j < n; j++) {
                    const int cj = next[j];
                    r += (cj < ck || (cj == ck && j < k));
                }
            }
            order[r] = k;
        }
        __syncwarp();
        bool unordered = false;
        for (int l = lane; l < n; l += 32) {
            const int k = order[l];
            const int64_t w2 = (int64_t)s * G + tv.sig[ab + k];
            // every list but level 0's must be in kd leaf order by now
            if (l > 0 && lstate && lstate[w2] != 2) unordered = true;
            lvl_off[l] = l == 0 ? cd.offset[w2] : cd.leaf_offset[w2];
            lvl_cnt[l] = cd.count[w2];
            tkey[l] = tv.key[ab + k];
            F[l] = 0;
            next[l] = 0;
            rem[l] = 0;
            cbase[l] = 0;
        }
        if (__any_sync(FULL_MASK, unordered)) {
            if (lane == 0) atomicMax(&counters[C_ERROR], 7ull);
            continue;
        }
        __syncwarp();
        const AnnulusParam *prm = tv.params + tv.param_begin[t];
        const double *tpos = tv.pos + 3 * (int64_t)ab;
        const int klast = order[n - 1];
        const int m0 = lvl_cnt[0];
        const int64_t off0 = lvl_off[0];
        int64_t emitted = 0, cut_base = 0;
        bool stop = false;
        const int64_t stop_at = (sa.best_match && sa.max_candidates >= 0) ? (int64_t)sa.max_candidates + 2 : -1;
        int lev = 0;
        while (!stop) {
            if ((++ticks & 255u) == 0) {
                int over = 0;
                if (lane == 0) over = (global_ns() - t_start) > sa.budget_ns;
                if (__shfl_sync(FULL_MASK, over, 0)) {
                    timed_out = true;
                    if (lane == 0) atomicMax(&counters[C_ERROR], 3ull);
                    break;
                }
            }
            if (lev == 0) {
                // next seed, in candidate order
                const int p = next[0];
                if (p >= m0) break;
                const int32_t a = cd.cand_atom[off0 + p];
                __syncwarp();
                if (lane == 0) {
                    next[0] = p + 1;
                    catom[0] = a;
                    ckey[0] = __float_as_int(cv.xyz32[abase + a].w);
                    trow[order[0]] = a;
                    F[0]++;
                    next[1] = 0;
                    rem[1] = 0;
                }
                __syncwarp();
                lev = 1;
                continue;
            }
            const bool last = lev == n - 1;
            if (!last && rem[lev]) {
                // the next passing leaf of the batch tested last
                const unsigned r = rem[lev];
                const int pos = cbase[lev] + __ffs(r) - 1;
                const int32_t a = cd.leaf_atom[lvl_off[lev] + pos];
                __syncwarp();
                if (lane == 0) {
                    rem[lev] = r & (r - 1);
                    catom[lev] = a;
                    ckey[lev] = __float_as_int(cv.xyz32[abase + a].w);
                    trow[order[lev]] = a;
                    next[lev + 1] = 0;
                    rem[lev + 1] = 0;
                }
                __syncwarp();
                lev++;
                continue;
            }
            const int mc = lvl_cnt[lev];
            const int base = next[lev];
            if (base >= mc) {
                lev--;
                continue;
            }
            // full test of leaf positions base .. base + 31
            const int p = base + lane;
            const int qn = order[lev];
            const int32_t tn = tkey[lev];
            bool pass = false;
            int32_t an = 0;
            if (p < mc) {
                an = cd.leaf_atom[lvl_off[lev] + p];
                const int32_t kn = __float_as_int(cv.xyz32[abase + an].w);
                pass = true;
                for (int j = 0; j < lev; j++)
                    if (!check_pair(ckey[j], kn, tkey[j], tn, sa.ignore_chain)) {
                        pass = false;
                        break;
                    }
                if (pass)
                    pass = decide_fp64_chain(lev - 1, catom, an, xyz64, prm, order, n, qn,
                                             cd.leaf_atom + lvl_off[lev], mc, p);
            }
            unsigned m = __ballot_sync(FULL_MASK, pass);
            __syncwarp();
            if (lane == 0) {
                F[lev] += __popc(m);
                next[lev] = base + 32;
                if (!last) {
                    rem[lev] = m;
                    cbase[lev] = base;
                }
            }
            __syncwarp();
            if (!last || !m) continue;
            // complete rows, in leaf order (Query.__next__'s max_candidates
            // cut applied inline in non-best mode, as in k_search)
            auto atom_of = [&](int k) -> int32_t { return k == klast ? an : trow[k]; };
            double rm = 0.0;
            if (sa.cut_inline) {
                bool hitf = false;
                if (pass) {
                    rm = lane_rmsd_by(n, atom_of, xyz64, tpos);
                    hitf = rm <= sa.rmsd_threshold && n >= 3;
                }
                const unsigned hl = __ballot_sync(FULL_MASK, hitf);
                unsigned mm = m;
                int r = 0, keep = 32;
                while (mm) {
                    const int ln = __ffs(mm) - 1;
                    mm &= mm - 1;
                    const int64_t q = emitted + r;
                    if (q - cut_base == (int64_t)sa.max_candidates + 1) {
                        keep = r;
                        stop = true;
                        break;
                    }
                    if ((hl >> ln) & 1u) cut_base = q + 1;
                    r++;
                }
                pass = pass && __popc(m & ((1u << lane) - 1u)) <= keep;
                m = __ballot_sync(FULL_MASK, pass);
            }
            const int np = __popc(m);
            int64_t row0 = 0;
            if (lane == 0) row0 = (int64_t)atomicAdd(out.count, (unsigned long long)np);
            row0 = __shfl_sync(FULL_MASK, row0, 0);
            if (pass) {
                const int rk = __popc(m & ((1u << lane) - 1u));
                const int64_t ri = row0 + rk;
                if (ri < out.capacity) {
                    int32_t *dst = out.atoms + ri * out.stride;
                    for (int k = 0; k < n; k++) dst[k] = atom_of(k);
                    out.pair[ri] = pair;
                    out.ordinal[ri] = emitted + rk;
                    if (out.rmsd) out.rmsd[ri] = rm;
                }
            }
            emitted += np;
            if (stop_at >= 0 && emitted >= stop_at) stop = true;
        }
        __syncwarp();
        if (lane == 0) {
            if (emitted > 0) out.pair_rows[pair] = (int32_t)emitted;
            int64_t partials = 0, bexp = 0;
            for (int l = 0; l < n; l++) partials += F[l];
            for (int l = 1; l < n; l++) bexp += 4LL * l * F[l - 1] + (4LL * (l + 1) + 16) * F[l];
            atomicAdd(&counters[C_PARTIALS], (unsigned long long)partials);
            atomicAdd(&counters[C_COMPLETE], (unsigned long long)F[n - 1]);
            atomicAdd(&counters[C_BYTES_EXP], (unsigned long long)bexp);
        }
        __syncwarp();
    }
}

// Superposition of every complete row, one thread per row (the FP64
// eigen-solve fills all lanes), written to the row's slot in reference
// order.
__global__ void k_superpose(ChunkView cv, TemplateView tv, CompleteRows in, RowResults out) {
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
    int64_t nrows = *in.count;
    if (nrows > in.capacity) nrows = in.capacity;
    const int T = tv.n_templates;
    for (int64_t i = tid; i < nrows; i += nthreads) {
        const int pair = in.pair[i];
        const int s = pair / T, t = pair % T;
        const int ab = tv.atom_begin[t];
        const int n = tv.atom_begin[t + 1] - ab;
        const double *xyz = cv.xyz64 + 3 * cv.atom_base[s];
        double ca[3], cb[3], S[9], E0;
        lane_covariance(n, in.atoms + i * in.stride, xyz, tv.pos + 3 * (int64_t)ab, ca, cb, S, &E0);
        double rmsd = 0.0, R[9];
        bool bad = false;
        quaternion_fit(S, E0, n, &rmsd, R, &bad);
        // rows whose rmsd already decided the max_candidates cut keep it, so
        // the automaton replays the same decisions
        if (in.rmsd) rmsd = in.rmsd[i];
        const int64_t d = out.off_q[(int64_t)s * T + (T - 1 - t)] + in.ordinal[i];
        out.rmsd[d] = rmsd;
        out.nan_rot[d] = bad ? 1 : 0;
        out.src[d] = i;
        for (int q = 0; q < 9; q++) out.rot[9 * d + q] = R[q];
        for (int k = 0; k < 3; k++) {
            out.centres[6 * d + k] = ca[k];
            out.centres[6 * d + 3 + k] = cb[k];
        }
    }
}

__global__ void k_order_counts(int64_t n_pairs, int32_t T, const int32_t *pair_rows, int32_t *cnt_q) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n_pairs) return;
    const int64_t s = q / T;
    const int t = T - 1 - (int)(q % T);
    cnt_q[q] = pair_rows[s * T + t];
}

// Query.__next__ (src/pyjess/_jess.pyx:2197-2283) in closed form, one
// thread per pair, over the pair's rows that pass the rmsd threshold:
//  best_match: over rows with ordinal <= M+1 (M = max_candidates), the
//    first strict minimum is the hit; a row with an undefined rotation that
//    would have lowered the minimum raises a warning instead.
//  otherwise: every passing row is a hit (an undefined rotation: a
//    warning), but the template's stream ends at the first row whose
//    ordinal is M+1 past the previous hit (or the template start).
__global__ void k_automaton(int64_t n_pairs, int32_t T, const int32_t *atom_begin, const int32_t *cnt_q,
                            const int64_t *off_q, RowResults rr, int32_t M, int32_t best, double thr, int32_t *hit,
                            int32_t *warn, int32_t *hit_atoms, unsigned long long *totals) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long nh = 0, nw = 0, na = 0, np = 0;
    if (q < n_pairs) {
        const int t = T - 1 - (int)(q % T);
        const int n = atom_begin[t + 1] - atom_begin[t];
        const int64_t off = off_q[q];
        const int64_t cnt = cnt_q[q];
        for (int64_t k = 0; k < cnt; k++) {
            hit[off + k] = 0;
            warn[off + k] = 0;
            hit_atoms[off + k] = 0;
        }
        if (best) {
            double cur = INFINITY;
            int64_t b = -1;
            for (int64_t k = 0; k < cnt; k++) {
                const double r = rr.rmsd[off + k];
                if (!(r <= thr)) continue;
                np++;
                if (M >= 0 && k > (int64_t)M + 1) break;
                if (r < cur) {
                    if (rr.nan_rot[off + k]) {
                        warn[off + k] = 1;
                        nw++;
                    } else {
                        cur = r;
                        b = k;
                    }
                }
            }
            if (b >= 0) {
                hit[off + b] = 1;
                hit_atoms[off + b] = n;
                nh++;
                na += n;
            }
        } else {
            int64_t base = 0;
            for (int64_t k = 0; k < cnt; k++) {
                const double r = rr.rmsd[off + k];
                if (!(r <= thr)) continue;
                np++;
                if (M >= 0 && k > base + M + 1) break;
                const bool nan_rot = rr.nan_rot[off + k] != 0;
                if (nan_rot) {
                    warn[off + k] = 1;
                    nw++;
                } else {
                    hit[off + k] = 1;
                    hit_atoms[off + k] = n;
                    nh++;
                    na += n;
                }
                if (M >= 0 && k == base + M + 1) break;
                if (!nan_rot) base = k + 1;
            }
        }
    }
    for (int o = 16; o; o >>= 1) {
        nh += __shfl_xor_sync(FULL_MASK, nh, o);
        nw += __shfl_xor_sync(FULL_MASK, nw, o);
        na += __shfl_xor_sync(FULL_MASK, na, o);
        np += __shfl_xor_sync(FULL_MASK, np, o);
    }
    if (lane_id() == 0) {
        if (nh) atomicAdd(&totals[0], nh);
        if (nw) atomicAdd(&totals[1], nw);
        if (na) atomicAdd(&totals[2], na);
        if (np) atomicAdd(&totals[3], np);
    }
}

// Flagged rows into the chunk's HitSegment, thread per row.
__global__ void k_gather_hits(int64_t n_rows, int32_t T, int32_t structure_base, int64_t atom_base,
                              const int32_t *atom_begin, CompleteRows in, RowResults rr, const int32_t *hit,
                              const int32_t *warn, const int64_t *hit_idx, const int64_t *warn_idx,
                              const int64_t *atom_idx, int32_t best, HitSegment out) {
    const int64_t d = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= n_rows) return;
    const bool h = hit[d] != 0, w = warn[d] != 0;
    if (!h && !w) return;
    const int64_t i = rr.src[d];
    const int pair = in.pair[i];
    const int s = pair / T, t = pair % T;
    const int64_t q = (int64_t)s * T + (T - 1 - t);
    if (h) {
        const int64_t k = hit_idx[d];
        out.structure[k] = structure_base + s;
        out.tpl[k] = t;
        out.ordinal[k] = in.ordinal[i];
        out.rmsd[k] = rr.rmsd[d];
        for (int c = 0; c < 9; c++) out.rot[9 * k + c] = rr.rot[9 * d + c];
        for (int c = 0; c < 6; c++) out.centres[6 * k + c] = rr.centres[6 * d + c];
        const int64_t a0 = atom_idx[d];
        out.atom_offset[k] = atom_base + a0;
        const int n = atom_begin[t + 1] - atom_begin[t];
        for (int j = 0; j < n; j++) out.atoms[a0 + j] = in.atoms[i * in.stride + j];
    }
    if (w) {
        const int64_t k = warn_idx[d];
        // hits of the structure already reported: best_match reports a
        // pair's hit after its rows, otherwise hits come in row order
        const int64_t first = hit_idx[rr.off_q[(int64_t)s * T]];
        const int64_t upto = best ? hit_idx[rr.off_q[q]] : hit_idx[d];
        out.warn_structure[k] = structure_base + s;
        out.warn_before[k] = upto - first;
    }
}

// ---------------------------------------------------------------------------
// Launchers

void launch_params(cudaStream_t st, int n_templates, const int32_t *atom_begin, const int32_t *param_begin,
                   const double *dist, const double *weight, double r, double s, double g, AnnulusParam *out) {
    if (n_templates > 0) k_params<<<n_templates, 256, 0, st>>>(n_templates, atom_begin, param_begin, dist, weight, r, s, g, out);
}

void launch_candidates(cudaStream_t st, int blocks, bool fill, const ChunkView &cv, const SigView &sv,
                       int32_t *count, int32_t *scanned, const int64_t *offset, int32_t *cand_atom,
                       const int64_t *work, const unsigned long long *n_work, int32_t *fill_state, bool claim) {
    if (fill)
        k_candidates<<<blocks, 256, 0, st>>>(cv, sv, offset, cand_atom, work, n_work, fill_state, claim ? 1 : 0);
    else {
        // thread per list
        const int64_t n = (int64_t)cv.n_structures * sv.n_sigs;
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const int cb = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)sms * 8));
        (void)blocks;
        k_candidate_counts<<<cb, 256, 0, st>>>(cv, sv, count, scanned);
    }
}

void launch_scan_tiles_i32(cudaStream_t st, const int32_t *in, int64_t n, int64_t *out, int64_t *tile_sums) {
    int64_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    k_scan_tiles<int32_t><<<(unsigned)tiles, SCAN_THREADS, 0, st>>>(in, n, out, tile_sums);
}

void launch_scan_tiles_i64(cudaStream_t st, const int64_t *in, int64_t n, int64_t *out, int64_t *tile_sums) {
    int64_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    k_scan_tiles<int64_t><<<(unsigned)tiles, SCAN_THREADS, 0, st>>>(in, n, out, tile_sums);
}

void launch_scan_add(cudaStream_t st, int64_t *out, int64_t n, const int64_t *tile_offsets) {
    k_scan_add<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(out, n, tile_offsets);
}

#if PJG_SEARCH_PROF
void leaf_profile_reset(cudaStream_t st) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_leaf_prof) == cudaSuccess)
        cudaMemsetAsync(p, 0, LP_NUM * sizeof(unsigned long long), st);
}

void leaf_profile_read(unsigned long long *h, cudaStream_t st) {
    cudaMemcpyFromSymbolAsync(h, g_leaf_prof, LP_NUM * sizeof(unsigned long long), 0, cudaMemcpyDeviceToHost, st);
}
#endif

void launch_leaf_order(cudaStream_t st, int blocks, const ChunkView &cv, int32_t n_sigs, const int32_t *count,
                       const int64_t *offset, const int64_t *blk_offset, const int32_t *cand_atom,
                       const int64_t *leaf_offset, int32_t *leaf_atom, float4 *leaf_xyz, float4 *blk_lo, float4 *blk_hi,
                       int64_t *sorted_list, unsigned long long *sorted_count, int64_t list_cap,
                       int64_t *exact_list, unsigned long long *exact_count, unsigned long long *counters,
                       const int64_t *work, const unsigned long long *n_work, int rank_max, uint8_t *part_ok,
                       int count_lists) {
    cudaMemsetAsync(sorted_count, 0, LEAF_LISTS * sizeof(unsigned long long), st);
    cudaMemsetAsync(exact_count, 0, sizeof(unsigned long long), st);
    rank_max = rank_max < 1 ? 1 : rank_max > LEAF_FAST_MAX ? LEAF_FAST_MAX : rank_max;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
#if PJG_LEAF_RANK
    // lists longer than rank_max go to the instance with larger buffers (up
    // to LEAF_MID_MAX entries), longer ones to the sorted-axis split
    int64_t *mid_list = sorted_list + 3 * list_cap;
    unsigned long long *mid_count = sorted_count + 3;
    k_leaf_order<LEAF_FAST_MAX, LEAF_WARPS><<<blocks, LEAF_WARPS * 32, 0, st>>>(
        cv, n_sigs, count, offset, blk_offset, cand_atom, leaf_offset, leaf_atom, leaf_xyz, blk_lo, blk_hi,
        sorted_list, sorted_count, list_cap, exact_list, exact_count, counters, rank_max, work, n_work, mid_list,
        mid_count, LEAF_MID_MAX, count_lists);
    (void)part_ok;
    k_leaf_order<LEAF_MID_MAX, 2><<<sms * 8, 64, 0, st>>>(
        cv, n_sigs, count, offset, blk_offset, cand_atom, leaf_offset, leaf_atom, leaf_xyz, blk_lo, blk_hi,
        sorted_list, sorted_count, list_cap, exact_list, exact_count, counters, LEAF_MID_MAX, mid_list, mid_count,
        nullptr, nullptr, 0, 0);
#else
    (void)blocks;
    // axis partitions: lists up to rank_max (<= 256 entries) in the first
    // instance (7 KB a warp, 4 warps a block), which forwards lists up to
    // 512 and 1024 entries to two instances with larger buffers (14 KB a
    // warp, 4 a block; 28 KB, 2 a block); one wave of resident blocks each
    int64_t *list512 = sorted_list + 3 * list_cap, *list1024 = sorted_list + 4 * list_cap;
    unsigned long long *count512 = sorted_count + 3, *count1024 = sorted_count + 4;
    auto wave = [&](const void *fn, int threads, int smem) {
        int per_sm = 0;
        cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem);
        return sms * (per_sm > 0 ? per_sm : 1);
    };
    {
        constexpr int SP = (int)sizeof(PartWarp<256>) * 4;
        const int g = wave((const void *)k_leaf_part<256, 4>, 128, SP);
        k_leaf_part<256, 4><<<g, 128, SP, st>>>(cv, n_sigs, count, offset, blk_offset, cand_atom, leaf_offset,
                                                leaf_atom, leaf_xyz, blk_lo, blk_hi, sorted_list, sorted_count,
                                                list_cap, exact_list, exact_count, counters, rank_max, work, n_work,
                                                PART_MAX >= 512 ? list512 : nullptr, count512, 512,
                                                PART_MAX >= 1024 ? list1024 : nullptr, count1024, 1024, count_lists,
                                                part_ok);
    }
    if (PART_MAX >= 512) {
        constexpr int SP = (int)sizeof(PartWarp<512>) * 4;
        const int g = wave((const void *)k_leaf_part<512, 4>, 128, SP);
        k_leaf_part<512, 4><<<g, 128, SP, st>>>(cv, n_sigs, count, offset, blk_offset, cand_atom, leaf_offset,
                                                leaf_atom, leaf_xyz, blk_lo, blk_hi, sorted_list, sorted_count,
                                                list_cap, exact_list, exact_count, counters, 512, list512, count512,
                                                nullptr, nullptr, 0, nullptr, nullptr, 0, 0, part_ok);
    }
    if (PART_MAX >= 1024) {
        constexpr int SP = (int)sizeof(PartWarp<1024>) * 2;
        const int g = wave((const void *)k_leaf_part<1024, 2>, 64, SP);
        k_leaf_part<1024, 2><<<g, 64, SP, st>>>(cv, n_sigs, count, offset, blk_offset, cand_atom, leaf_offset,
                                                leaf_atom, leaf_xyz, blk_lo, blk_hi, sorted_list, sorted_count,
                                                list_cap, exact_list, exact_count, counters, 1024, list1024,
                                                count1024, nullptr, nullptr, 0, nullptr, nullptr, 0, 0, part_ok);
    }
#endif
    // sorted-axis split, one worklist per size class: up to 512 entries
    // 13 KB a warp (4 warps a block), up to 1024 25 KB (2 a block), up to
    // LEAF_SORTED_MAX 50 KB (1 a block)
    constexpr int SS0 = (int)sizeof(SortedWarp<512>) * 4;
    cudaFuncSetAttribute(k_leaf_sorted<512, 0, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, SS0);
    k_leaf_sorted<512, 0, 4><<<sms * 4, 128, SS0, st>>>(cv, n_sigs, count, offset, blk_offset, cand_atom, leaf_offset,
                                                       leaf_atom, leaf_xyz, blk_lo, blk_hi, sorted_list,
                                                       sorted_count, exact_list, exact_count, counters);
    constexpr int SS1 = (int)sizeof(SortedWarp<1024>) * 2;
    cudaFuncSetAttribute(k_leaf_sorted<1024, 512, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, SS1);
    k_leaf_sorted<1024, 512, 2><<<sms * 4, 64, SS1, st>>>(cv, n_sigs, count, offset, blk_offset, cand_atom,
                                                         leaf_offset, leaf_atom, leaf_xyz, blk_lo, blk_hi,
                                                         sorted_list + list_cap, sorted_count + 1, exact_list,
                                                         exact_count, counters);
    constexpr int SS2 = (int)sizeof(SortedWarp<LEAF_SORTED_MAX>);
    cudaFuncSetAttribute(k_leaf_sorted<LEAF_SORTED_MAX, 1024, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, SS2);
    k_leaf_sorted<LEAF_SORTED_MAX, 1024, 1><<<sms * 4, 32, SS2, st>>>(
        cv, n_sigs, count, offset, blk_offset, cand_atom, leaf_offset, leaf_atom, leaf_xyz, blk_lo, blk_hi,
        sorted_list + 2 * list_cap, sorted_count + 2, exact_list, exact_count, counters);
    // exact replay: lists up to 1024 entries 16 KB a warp, 4 warps a block
    constexpr int SM1 = 1024 * 16 * 4;
    cudaFuncSetAttribute(k_leaf_exact<1024, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, SM1);
    k_leaf_exact<1024, 0><<<sms * 3, 128, SM1, st>>>(cv, n_sigs, count, offset, blk_offset, cand_atom, leaf_offset,
                                                    leaf_atom, leaf_xyz, blk_lo, blk_hi, exact_list, exact_count,
                                                    counters);
    // longer lists: 64 KB a warp, one warp a block (beyond EXACT_MAX: one
    // thread replays the list from global memory)
    constexpr int SM2 = EXACT_MAX * 16;
    cudaFuncSetAttribute(k_leaf_exact<EXACT_MAX, 1024>, cudaFuncAttributeMaxDynamicSharedMemorySize, SM2);
    k_leaf_exact<EXACT_MAX, 1024><<<sms * 3, 32, SM2, st>>>(cv, n_sigs, count, offset, blk_offset, cand_atom,
                                                           leaf_offset, leaf_atom, leaf_xyz, blk_lo, blk_hi,
                                                           exact_list, exact_count, counters);
}

void launch_axis_ranks(cudaStream_t st, int32_t n_structures, const int64_t *atom_base, const int32_t *atom_count,
                       const double *xyz64, int64_t n_atoms, unsigned long long *tile_key, uint16_t *tile_idx,
                       uint32_t *lrank, uint32_t *urank) {
    if (n_structures <= 0) return;
    k_axis_ranks<<<dim3((unsigned)n_structures, 3), RANK_THREADS, 0, st>>>(atom_base, atom_count, xyz64, n_atoms,
                                                                          tile_key, tile_idx, lrank, urank);
}

void launch_demand_levels(cudaStream_t st, int blocks, const TemplateView &tv, const CandView &cd, int32_t n_pairs,
                          int32_t max_level, int32_t reorder, const LeafDemand &dm) {
    // (also with max_level 0: the pairs of templates over 32 atoms request
    // every list here)
    // thread per pair
    (void)blocks;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int g = (int)std::max<int64_t>(1, std::min<int64_t>(((int64_t)n_pairs + 255) / 256, (int64_t)sms * 8));
    if (n_pairs > 0) k_demand_levels<<<g, 256, 0, st>>>(tv, cd, n_pairs, max_level, reorder, dm);
}

void launch_list_keys(cudaStream_t st, int blocks, int32_t n_sigs, const int32_t *count, const int64_t *offset,
                      const int32_t *cand_atom, const int64_t *work, const unsigned long long *n_work,
                      const ListShare &ls, unsigned long long *counters) {
    k_list_keys<<<blocks, 256, 0, st>>>(n_sigs, count, offset, cand_atom, work, n_work, ls, counters);
}

void launch_list_reps(cudaStream_t st, int blocks, const int64_t *work, const unsigned long long *n_work,
                      const ListShare &ls) {
    k_list_reps<<<blocks, 256, 0, st>>>(work, n_work, ls);
}

void launch_list_share(cudaStream_t st, int blocks, const ChunkView &cv, int32_t n_sigs, const int32_t *count,
                       const int64_t *offset, const int32_t *cand_atom, int64_t *leaf_offset, int64_t *blk_offset,
                       const ListShare &ls, unsigned long long *counters) {
    k_list_share<8><<<blocks, 256, 0, st>>>(cv, n_sigs, count, offset, cand_atom, leaf_offset, blk_offset, ls,
                                            counters);
}

void launch_heavy_pairs(cudaStream_t st, int32_t n_pairs, const uint8_t *pair_cost, unsigned long long *bins,
                        int64_t target, uint8_t *heavy_flag, int32_t *heavy) {
    if (n_pairs <= 0) return;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int g = (int)std::max<int64_t>(1, std::min<int64_t>(((int64_t)n_pairs + 255) / 256, (int64_t)sms * 4));
    k_cost_hist<<<g, 256, 0, st>>>(n_pairs, pair_cost, bins);
    k_heavy_list<<<g, 256, 0, st>>>(n_pairs, pair_cost, bins, target, heavy_flag, heavy);
}

void launch_mark_ordered(cudaStream_t st, int blocks, const LeafDemand &dm) {
    k_mark_ordered<<<blocks, 256, 0, st>>>(dm);
}

void launch_block_counts(cudaStream_t st, int64_t n, const int32_t *count, int32_t *nblk) {
    if (n > 0) k_block_counts<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, count, nblk);
}

template <typename RowT, bool FP32, bool CUT>
static cudaError_t search_variant(cudaStream_t st, int grid, const ChunkView &cv, const TemplateView &tv,
                                  const CandView &cd, const SearchArgs &sa, int32_t *pair_counter,
                                  const int32_t *scanned, const CompleteRows &out, unsigned long long *counters,
                                  const LeafDemand &dm) {
    size_t smem = (size_t)sa.warp_smem * SEARCH_WARPS;
    auto kern = k_search<RowT, FP32, CUT>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    // persistent grid: as many blocks as can be resident at once
    int per_sm = 0, dev = 0, sms = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, SEARCH_WARPS * 32, smem);
    if (e != cudaSuccess) return e;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (per_sm > 0 && sms > 0) grid = per_sm * sms;
    kern<<<grid, SEARCH_WARPS * 32, smem, st>>>(cv, tv, cd, sa, pair_counter, scanned, out, counters, dm);
    return cudaGetLastError();
}

template <typename RowT, bool FP32>
static cudaError_t search_cut(cudaStream_t st, int grid, const ChunkView &cv, const TemplateView &tv,
                              const CandView &cd, const SearchArgs &sa, int32_t *pair_counter, const int32_t *scanned,
                              const CompleteRows &out, unsigned long long *counters, const LeafDemand &dm) {
    return sa.cut_inline
               ? search_variant<RowT, FP32, true>(st, grid, cv, tv, cd, sa, pair_counter, scanned, out, counters, dm)
               : search_variant<RowT, FP32, false>(st, grid, cv, tv, cd, sa, pair_counter, scanned, out, counters, dm);
}

#if PJG_SEARCH_PROF
__global__ void k_prof_tail(unsigned long long *prof) {
    if (g_search_tail[1] > g_search_tail[0]) prof[SP_TAIL_NS] += g_search_tail[1] - g_search_tail[0];
}
#endif

cudaError_t launch_search(cudaStream_t st, int grid, bool wide, bool fp32, const ChunkView &cv,
                          const TemplateView &tv, const CandView &cd, const SearchArgs &sa, int32_t *pair_counter,
                          const int32_t *scanned, const CompleteRows &out, unsigned long long *counters,
                          const LeafDemand &dm) {
#if PJG_SEARCH_PROF
    const unsigned long long t0[2] = {~0ull, 0ull};
    cudaMemcpyToSymbolAsync(g_search_tail, t0, sizeof t0, 0, cudaMemcpyHostToDevice, st);
#endif
    cudaError_t e;
    if (wide)
        e = fp32 ? search_cut<uint32_t, true>(st, grid, cv, tv, cd, sa, pair_counter, scanned, out, counters, dm)
                 : search_cut<uint32_t, false>(st, grid, cv, tv, cd, sa, pair_counter, scanned, out, counters, dm);
    else
        e = fp32 ? search_cut<uint16_t, true>(st, grid, cv, tv, cd, sa, pair_counter, scanned, out, counters, dm)
                 : search_cut<uint16_t, false>(st, grid, cv, tv, cd, sa, pair_counter, scanned, out, counters, dm);
#if PJG_SEARCH_PROF
    if (e == cudaSuccess && sa.prof) k_prof_tail<<<1, 1, 0, st>>>(sa.prof);
#endif
    return e;
}

cudaError_t launch_search_large(cudaStream_t st, const ChunkView &cv, const TemplateView &tv, const CandView &cd,
                                const SearchArgs &sa, const int32_t *large, int32_t n_large, int32_t *item_counter,
                                const int32_t *scanned, const CompleteRows &out, unsigned long long *counters,
                                const int32_t *lstate) {
    if (n_large <= 0 || cv.n_structures <= 0) return cudaSuccess;
    const size_t smem = (size_t)large_warp_bytes(tv.max_atoms) * LARGE_WARPS;
    cudaError_t e = cudaFuncSetAttribute(k_search_large, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t items = (int64_t)cv.n_structures * n_large;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((items + LARGE_WARPS - 1) / LARGE_WARPS,
                                                                 (int64_t)std::max(sms, 1) * 4));
    k_search_large<<<grid, LARGE_WARPS * 32, smem, st>>>(cv, tv, cd, sa, large, n_large, item_counter, scanned, out,
                                                         counters, lstate);
    return cudaGetLastError();
}

// Hit atoms in the template frame: thread per hit, each of its matched
// molecule atoms x mapped by the hit's transformation T(v) R T(-c)
// (Hit.transformation, src/pyjess/_jess.pyx:2343-2377): R x + t with
// t = R (-c) + v.
__global__ void k_superposed_atoms(int64_t n_hits, int64_t n_atoms, const int32_t *structure,
                                   const int64_t *atom_offset, const int32_t *atoms, const double *rot,
                                   const double *centres, const int64_t *atom_base, const double *xyz64,
                                   double *out) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; h < n_hits; h += stride) {
        const double *R = rot + 9 * h;
        const double *c = centres + 6 * h;
        double t[3];
        for (int i = 0; i < 3; i++) {
            double acc = __dmul_rn(R[3 * i], -c[0]);
            acc = __dadd_rn(acc, __dmul_rn(R[3 * i + 1], -c[1]));
            acc = __dadd_rn(acc, __dmul_rn(R[3 * i + 2], -c[2]));
            t[i] = __dadd_rn(acc, c[3 + i]);
        }
        const double *xs = xyz64 + 3 * atom_base[structure[h]];
        // the hit store holds the first atom of each hit; the last hit ends
        // at the store's atom count
        const int64_t k1 = h + 1 < n_hits ? atom_offset[h + 1] : n_atoms;
        for (int64_t k = atom_offset[h]; k < k1; k++) {
            const double *x = xs + 3 * (int64_t)atoms[k];
            for (int i = 0; i < 3; i++) {
                double acc = __dmul_rn(R[3 * i], x[0]);
                acc = __dadd_rn(acc, __dmul_rn(R[3 * i + 1], x[1]));
                acc = __dadd_rn(acc, __dmul_rn(R[3 * i + 2], x[2]));
                out[3 * k + i] = __dadd_rn(acc, t[i]);
            }
        }
    }
}

void launch_superposed_atoms(cudaStream_t st, int64_t n_hits, int64_t n_atoms, const int32_t *structure,
                             const int64_t *atom_offset, const int32_t *atoms, const double *rot,
                             const double *centres, const int64_t *atom_base, const double *xyz64, double *out) {
    if (n_hits <= 0) return;
    const int blocks = (int)std::min<int64_t>((n_hits + 255) / 256, 152 * 32);
    k_superposed_atoms<<<blocks, 256, 0, st>>>(n_hits, n_atoms, structure, atom_offset, atoms, rot, centres,
                                               atom_base, xyz64, out);
}

void launch_superpose(cudaStream_t st, int blocks, const ChunkView &cv, const TemplateView &tv,
                      const CompleteRows &in, const RowResults &out) {
    k_superpose<<<blocks, 128, 0, st>>>(cv, tv, in, out);
}

void launch_order_counts(cudaStream_t st, int64_t n_pairs, int32_t n_templates, const int32_t *pair_rows,
                         int32_t *cnt_q) {
    if (n_pairs > 0)
        k_order_counts<<<(unsigned)((n_pairs + 255) / 256), 256, 0, st>>>(n_pairs, n_templates, pair_rows, cnt_q);
}

void launch_automaton(cudaStream_t st, int64_t n_pairs, int32_t n_templates, const int32_t *atom_begin,
                      const int32_t *cnt_q, const int64_t *off_q, const RowResults &rr, int32_t max_candidates,
                      int32_t best_match, double rmsd_threshold, int32_t *hit, int32_t *warn, int32_t *hit_atoms,
                      unsigned long long *totals) {
    if (n_pairs > 0)
        k_automaton<<<(unsigned)((n_pairs + 127) / 128), 128, 0, st>>>(n_pairs, n_templates, atom_begin, cnt_q,
                                                                      off_q, rr, max_candidates, best_match,
                                                                      rmsd_threshold, hit, warn, hit_atoms, totals);
}

void launch_gather_hits(cudaStream_t st, int64_t n_rows, int32_t n_templates, int32_t structure_base,
                        int64_t atom_base, const int32_t *atom_begin, const CompleteRows &in, const RowResults &rr,
                        const int32_t *hit, const int32_t *warn, const int64_t *hit_idx, const int64_t *warn_idx,
                        const int64_t *atom_idx, int32_t best_match, const HitSegment &out) {
    if (n_rows > 0)
        k_gather_hits<<<(unsigned)((n_rows + 255) / 256), 256, 0, st>>>(n_rows, n_templates, structure_base,
                                                                        atom_base, atom_begin, in, rr, hit, warn,
                                                                        hit_idx, warn_idx, atom_idx, best_match, out);
}

// ---------------------------------------------------------------------------
// Superposition without allocation (pjg_superpose_noalloc).
//
// For callers that cannot allocate device memory while they run -- a
// real-time loop that must not block on the allocator, or a host
// application whose memory manager owns every device allocation -- this variant of k_superpose takes the assignments' molecule
// coordinates and the template's coordinates directly from the caller,
// writes the caller's output arrays, and keeps its only scratch (one pass
// flag per row, for the order-preserving compaction of the rows under the
// rmsd threshold) in the static array below.  The array is part of the
// library image: every GPU that loads the library holds it until the process
// exits.  Every call shares it, so calls that overlap on the GPU (other
// streams, other host threads) race and must be serialised by the caller.
// Each call writes the flag of every row it later reads, so nothing carries
// over from one call to the next.

static __device__ __align__(256) int32_t g_noalloc_flags[PJG_NOALLOC_MAX_ROWS];

__global__ void k_superpose_rows(const double *mol_xyz, const double *tpl_xyz, int32_t n_rows, int32_t n,
                                 double rmsd_threshold, double *rmsd_out, double *rot_out, double *cen_out,
                                 int32_t *flags) {
    const int lane = lane_id();
    int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = warp; i < n_rows; i += nwarps) {
        double a[3] = {0, 0, 0}, b[3] = {0, 0, 0};
        if (lane < n) {
            for (int d = 0; d < 3; d++) {
                a[d] = mol_xyz[(i * n + lane) * 3 + d];
                b[d] = tpl_xyz[3 * lane + d];
            }
        }
        double ca[3], cb[3];
        for (int d = 0; d < 3; d++) {
            ca[d] = warp_sum(a[d]) / (double)n;
            cb[d] = warp_sum(b[d]) / (double)n;
        }
        double ac[3] = {0, 0, 0}, bc[3] = {0, 0, 0};
        if (lane < n)
            for (int d = 0; d < 3; d++) {
                ac[d] = a[d] - ca[d];
                bc[d] = b[d] - cb[d];
            }
        double sumA = warp_sum(ac[0] * ac[0] + ac[1] * ac[1] + ac[2] * ac[2]);
        double sumB = warp_sum(bc[0] * bc[0] + bc[1] * bc[1] + bc[2] * bc[2]);
        double S[9];
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) S[3 * r + c] = warp_sum(ac[r] * bc[c]);
        if (lane == 0) {
            double rmsd = 0.0, R[9];
            bool bad = false;
            quaternion_fit(S, 0.5 * (sumA + sumB), n, &rmsd, R, &bad);
            rmsd_out[i] = rmsd;
            for (int q = 0; q < 9; q++) rot_out[9 * i + q] = R[q];
            for (int d = 0; d < 3; d++) {
                cen_out[6 * i + d] = ca[d];
                cen_out[6 * i + 3 + d] = cb[d];
            }
            flags[i] = (rmsd <= rmsd_threshold && !bad) ? 1 : 0;
        }
    }
}

// one block: rows whose flag is set, in row order, and their count
__global__ void k_compact_rows(const int32_t *flags, int32_t n_rows, int32_t *pass_rows, int32_t *pass_count) {
    __shared__ int32_t warp_tot[32];
    const int lane = lane_id(), wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int32_t base = 0;
    for (int32_t t0 = 0; t0 < n_rows; t0 += blockDim.x) {
        const int32_t i = t0 + threadIdx.x;
        const bool f = i < n_rows && flags[i] != 0;
        const unsigned m = __ballot_sync(FULL_MASK, f);
        if (lane == 0) warp_tot[wid] = __popc(m);
        __syncthreads();
        int32_t before = 0, total = 0;
        for (int w = 0; w < nw; w++) {
            if (w < wid) before += warp_tot[w];
            total += warp_tot[w];
        }
        if (f) pass_rows[base + before + __popc(m & ((1u << lane) - 1u))] = i;
        base += total;
        __syncthreads();
    }
    if (threadIdx.x == 0) *pass_count = base;
}

}  // namespace pjg

// ---------------------------------------------------------------------------
// C entry point of the allocation-free superposition

#include <mutex>

#include "../../include/pjg.h"

namespace {
std::mutex g_noalloc_mutex;
void *g_noalloc_ptr[64] = {};                 // device address of g_noalloc_flags, per device
unsigned long long g_noalloc_ctx[64] = {};    // id of the context that address belongs to
thread_local char g_noalloc_err[256];

// Unique id of the calling thread's current CUDA context (0 if unknown).
// The driver never reuses an id, so a context destroyed and recreated on
// the same device (cudaDeviceReset, then new work) gets a new one.  The two
// driver calls are reached through the runtime's entry-point query, so the
// library needs no link against the driver library.
unsigned long long current_context_id() {
    using GetCurrent = int (*)(void **);
    using GetId = int (*)(void *, unsigned long long *);
    static GetCurrent get_current = [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            f = nullptr;
        cudaGetLastError();
        return (GetCurrent)f;
    }();
    static GetId get_id = [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            f = nullptr;
        cudaGetLastError();
        return (GetId)f;
    }();
    void *ctx = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0;
    return id;
}
}  // namespace

extern "C" const char *pjg_noalloc_last_error(void) { return g_noalloc_err; }

// No counterpart in the reference: see include/pjg.h.
extern "C" pjg_status pjg_superpose_noalloc(const double *mol_xyz, const double *tpl_xyz, int32_t n_rows,
                                            int32_t n_atoms, double rmsd_threshold, double *rmsd, double *rotation,
                                            double *centres, int32_t *pass_rows, int32_t *pass_count,
                                            void *stream) {
    g_noalloc_err[0] = 0;
    if (n_rows < 0 || n_rows > PJG_NOALLOC_MAX_ROWS) {
        snprintf(g_noalloc_err, sizeof g_noalloc_err,
                 "pjg_superpose_noalloc: %d rows requested, the static scratch holds at most %d", n_rows,
                 PJG_NOALLOC_MAX_ROWS);
        return PJG_ERR_INVALID;
    }
    if (n_atoms < 1 || n_atoms > 32) {
        snprintf(g_noalloc_err, sizeof g_noalloc_err, "pjg_superpose_noalloc: %d atoms per row (1 to 32 allowed)",
                 n_atoms);
        return PJG_ERR_INVALID;
    }
    if (!pass_count || (n_rows > 0 && (!mol_xyz || !tpl_xyz || !rmsd || !rotation || !centres || !pass_rows))) {
        snprintf(g_noalloc_err, sizeof g_noalloc_err, "pjg_superpose_noalloc: null pointer argument");
        return PJG_ERR_INVALID;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= 64) {
        snprintf(g_noalloc_err, sizeof g_noalloc_err, "pjg_superpose_noalloc: no current device (%s)",
                 cudaGetErrorString(e));
        return PJG_ERR_NO_DEVICE;
    }
    void *flags = nullptr;
    {
        // once per device and context, with that device current: the device
        // address of the static scratch (host code must not pass the symbol
        // itself).  A context reset since the lookup (a new context id) gets
        // the address looked up again, so a cached address is never used in
        // a context it does not belong to.  (Before the process's first
        // CUDA call there is no context yet: the lookup creates it, and the
        // id is read after it.)
        const unsigned long long ctx = current_context_id();
        std::lock_guard<std::mutex> lock(g_noalloc_mutex);
        if (!g_noalloc_ptr[dev] || ctx == 0 || ctx != g_noalloc_ctx[dev]) {
            void *p = nullptr;
            e = cudaGetSymbolAddress(&p, pjg::g_noalloc_flags);
            if (e != cudaSuccess || !p) {
                snprintf(g_noalloc_err, sizeof g_noalloc_err, "pjg_superpose_noalloc: cudaGetSymbolAddress: %s",
                         cudaGetErrorString(e));
                return PJG_ERR_CUDA;
            }
            g_noalloc_ptr[dev] = p;
            g_noalloc_ctx[dev] = current_context_id();
        }
        flags = g_noalloc_ptr[dev];
    }
    cudaStream_t st = (cudaStream_t)stream;
    if (n_rows > 0) {
        int blocks = (int)std::min<int64_t>(((int64_t)n_rows + 7) / 8, 4096);
        pjg::k_superpose_rows<<<blocks, 256, 0, st>>>(mol_xyz, tpl_xyz, n_rows, n_atoms, rmsd_threshold, rmsd,
                                                      rotation, centres, (int32_t *)flags);
    }
    pjg::k_compact_rows<<<1, 1024, 0, st>>>((const int32_t *)flags, n_rows, pass_rows, pass_count);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        snprintf(g_noalloc_err, sizeof g_noalloc_err, "pjg_superpose_noalloc: launch: %s", cudaGetErrorString(e));
        return PJG_ERR_CUDA;
    }
    return PJG_OK;
}
