// pjg_api.cu — C ABI of libpjg (include/pjg.h): template / structure
// upload and the query pipeline.
//
// Pipeline of pjg_query (on one CUDA stream owned by the call):
//   k_params                      annulus radii for the query's r and s
//   k_candidate_counts            |C| and |R| of every (structure, signature)
//   k_struct_totals               candidate entries per structure
//   per structure chunk (bounded entry budget):
//     k_scan_*, k_block_counts    list offsets, culling blocks of CULL_BLK leaves
//     k_candidates                lists in candidate order
//     k_demand_levels             requests the lists of the first levels
//     k_leaf_order, k_leaf_sorted, k_leaf_exact, k_mark_ordered
//                                 requested lists in kd leaf order
//     k_search                    complete assignments, ordered per pair;
//                                 pairs that reach a list without leaf order
//                                 request it and are suspended, the lists are
//                                 ordered (as above) and a second k_search
//                                 round resumes them
//     k_superpose                 rmsd / rotation / centroids per row
//     k_order_counts, k_automaton, k_gather_hits
//                                 rows in (structure, template descending,
//                                 ordinal) order, the Query.__next__
//                                 automaton (src/pyjess/_jess.pyx:2197-2283)
//                                 per pair, hits and warnings compacted

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <unordered_map>
#include <mutex>
#include <numeric>
#include <atomic>
#include <string>
#include <thread>
#include <vector>

#include "../../include/pjg.h"
#include "pjg_common.cuh"
#include "pjg_kernels.cuh"

using namespace pjg;

namespace {

thread_local std::string g_error = "";

pjg_status fail(pjg_status st, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_error = buf;
    return st;
}

#define CUDA_TRY(expr)                                                                          \
    do {                                                                                        \
        cudaError_t _e = (expr);                                                                \
        if (_e != cudaSuccess) {                                                                \
            status = fail(_e == cudaErrorMemoryAllocation ? PJG_ERR_OOM : PJG_ERR_CUDA,         \
                          "%s failed: %s (%s:%d)", #expr, cudaGetErrorString(_e), __FILE__,     \
                          __LINE__);                                                            \
            goto done;                                                                          \
        }                                                                                       \
    } while (0)

inline uint8_t up(uint8_t c) { return (c >= 'a' && c <= 'z') ? (uint8_t)(c & ~0x20) : c; }

inline uint32_t pack_upper(const uint8_t *b) {
    return (uint32_t)up(b[0]) | ((uint32_t)up(b[1]) << 8) | ((uint32_t)up(b[2]) << 16) |
           ((uint32_t)up(b[3]) << 24);
}

inline uint32_t pack_lit(const char *s) { return pack_upper((const uint8_t *)s); }

// device buffer helper (stream ordered)
template <typename T>
struct DBuf {
    T *p = nullptr;
    size_t n = 0;
};

template <typename T>
cudaError_t dalloc(DBuf<T> &b, size_t n, cudaStream_t st) {
    if (b.n >= n && b.p) return cudaSuccess;
    if (b.p) cudaFreeAsync(b.p, st);
    b.p = nullptr;
    b.n = 0;
    size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
    cudaError_t e = cudaMallocAsync((void **)&b.p, bytes, st);
    if (e == cudaSuccess) b.n = std::max<size_t>(n, 1);
    return e;
}

template <typename T>
void dfree(DBuf<T> &b, cudaStream_t st) {
    if (b.p) cudaFreeAsync(b.p, st);
    b.p = nullptr;
    b.n = 0;
}

template <typename T>
cudaError_t upload(T **dst, const T *src, size_t n) {
    cudaError_t e = cudaMalloc((void **)dst, std::max<size_t>(n, 1) * sizeof(T));
    if (e != cudaSuccess) return e;
    if (n) e = cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice);
    return e;
}

template <typename T>
cudaError_t upload(T **dst, const std::vector<T> &v) {
    return upload(dst, v.data(), v.size());
}

// Host staging array of n elements left uninitialised (every element is
// written before use; a std::vector would zero it first).
template <typename T>
struct HostArray {
    std::unique_ptr<T[]> p;
    explicit HostArray(size_t n) : p(new T[std::max<size_t>(n, 1)]) {}
    T &operator[](size_t i) { return p[i]; }
    const T &operator[](size_t i) const { return p[i]; }
};

// Chemically equivalent atom pairs used by match mode 1 (see the oracle's
// same_position rule; pinned by the reference fixture for ASN OD1/ND2).
struct PartnerDef { const char *res; const char *a; const char *b; };
const PartnerDef PARTNER_TABLE[] = {
    {"ASP", "_OD1", "_OD2"}, {"GLU", "_OE1", "_OE2"}, {"ASN", "_OD1", "_ND2"},
    {"GLN", "_OE1", "_NE2"}, {"ARG", "_NH1", "_NH2"}, {"HIS", "_ND1", "_CD2"},
    {"HIS", "_CE1", "_NE2"}, {"PHE", "_CD1", "_CD2"}, {"PHE", "_CE1", "_CE2"},
    {"TYR", "_CD1", "_CD2"}, {"TYR", "_CE1", "_CE2"}, {"LEU", "_CD1", "_CD2"},
    {"VAL", "_CG1", "_CG2"},
};

uint32_t res_lit(const char *three) {
    uint8_t b[4] = {(uint8_t)three[0], (uint8_t)three[1], (uint8_t)three[2], 0};
    return pack_upper(b);
}

}  // namespace

// ---------------------------------------------------------------------------
// Handles

struct pjg_templates {
    int32_t T = 0, A = 0, nmax = 0, G = 0;
    std::vector<int32_t> atom_begin, param_begin, dim;
    // device
    int32_t *d_atom_begin = nullptr, *d_sig = nullptr, *d_key = nullptr, *d_param_begin = nullptr;
    double *d_pos = nullptr, *d_weight = nullptr, *d_dist = nullptr;
    int32_t *d_code = nullptr, *d_rule = nullptr, *d_mainchain = nullptr, *d_name_begin = nullptr,
            *d_res_begin = nullptr, *d_partner_begin = nullptr;
    uint32_t *d_names = nullptr, *d_resnames = nullptr, *d_partner_res = nullptr, *d_partner_name = nullptr;
    int64_t n_params = 0;
    int device = 0;
    // templates of more than 32 atoms (searched by k_search_large)
    std::vector<int32_t> large;
    int32_t *d_large = nullptr;
};

struct pjg_structures {
    int32_t S = 0;
    int64_t N = 0;
    int32_t max_atoms = 0;
    double max_radius = 0.0;
    std::vector<int64_t> atom_base;
    int64_t *d_atom_base = nullptr;
    int32_t *d_atom_count = nullptr;
    double *d_xyz64 = nullptr;
    float4 *d_xyz32 = nullptr;
    uint32_t *d_name = nullptr, *d_resname = nullptr;
    int32_t *d_sorted = nullptr;
    int32_t *d_bucket_begin = nullptr, *d_bucket_lo = nullptr, *d_bucket_hi = nullptr;
    uint32_t *d_bucket_name = nullptr;
    uint32_t *d_lrank = nullptr, *d_urank = nullptr;  // [3][N] axis ranks
    int32_t *d_nh_begin = nullptr, *d_nh_count = nullptr;  // name histogram per bucket
    uint32_t *d_nh_name = nullptr;
    uint8_t *d_name_id = nullptr;                      // name index within the bucket
    // per distinct name of a bucket: where its atoms start (structure-local)
    // in nh_pos, which holds every structure's atoms grouped by (bucket,
    // name), each group in ResIndex order
    int32_t *d_nh_off = nullptr, *d_nh_pos = nullptr;
    int device = 0;
};

// Hits and warnings of a query, on the device: contiguous arrays that grow
// (doubling) as chunks append to them.
struct HitStore {
    int64_t hits = 0, atoms = 0, warns = 0;           // in use
    int64_t cap_h = 0, cap_a = 0, cap_w = 0;          // allocated
    int32_t *structure = nullptr, *tpl = nullptr, *atoms_ = nullptr, *warn_structure = nullptr;
    int64_t *ordinal = nullptr, *atom_offset = nullptr, *warn_before = nullptr;
    double *rmsd = nullptr, *rot = nullptr, *centres = nullptr;

    template <typename T>
    static cudaError_t grow(T **p, int64_t used, int64_t cap, int64_t width, cudaStream_t st) {
        T *q = nullptr;
        cudaError_t e = cudaMalloc((void **)&q, (size_t)std::max<int64_t>(cap, 1) * width * sizeof(T));
        if (e != cudaSuccess) return e;
        if (*p && used > 0) e = cudaMemcpyAsync(q, *p, (size_t)used * width * sizeof(T), cudaMemcpyDeviceToDevice, st);
        if (*p) {
            cudaStreamSynchronize(st);
            cudaFree(*p);
        }
        *p = q;
        return e;
    }
    // room for `h` more hits, `a` more atoms, `w` more warnings
    cudaError_t reserve(int64_t h, int64_t a, int64_t w, cudaStream_t st) {
        cudaError_t e = cudaSuccess;
        if (hits + h > cap_h) {
            int64_t c = std::max<int64_t>(hits + h, 2 * cap_h);
            if (e == cudaSuccess) e = grow(&structure, hits, c, 1, st);
            if (e == cudaSuccess) e = grow(&tpl, hits, c, 1, st);
            if (e == cudaSuccess) e = grow(&ordinal, hits, c, 1, st);
            if (e == cudaSuccess) e = grow(&atom_offset, hits, c + 1, 1, st);
            if (e == cudaSuccess) e = grow(&rmsd, hits, c, 1, st);
            if (e == cudaSuccess) e = grow(&rot, hits, c, 9, st);
            if (e == cudaSuccess) e = grow(&centres, hits, c, 6, st);
            if (e == cudaSuccess) cap_h = c;
        }
        if (atoms + a > cap_a && e == cudaSuccess) {
            int64_t c = std::max<int64_t>(atoms + a, 2 * cap_a);
            e = grow(&atoms_, atoms, c, 1, st);
            if (e == cudaSuccess) cap_a = c;
        }
        if (warns + w > cap_w && e == cudaSuccess) {
            int64_t c = std::max<int64_t>(warns + w, 2 * cap_w);
            e = grow(&warn_structure, warns, c, 1, st);
            if (e == cudaSuccess) e = grow(&warn_before, warns, c, 1, st);
            if (e == cudaSuccess) cap_w = c;
        }
        return e;
    }
    // the segment view at the current ends
    HitSegment tail() const {
        return HitSegment{structure + hits, tpl + hits, ordinal + hits, rmsd + hits, rot + 9 * hits,
                          centres + 6 * hits, atom_offset + hits, atoms_ + atoms, warn_structure + warns,
                          warn_before + warns};
    }
    ~HitStore() {
        void *ptrs[] = {structure, tpl, atoms_, warn_structure, ordinal, atom_offset, warn_before, rmsd, rot, centres};
        for (void *p : ptrs)
            if (p) cudaFree(p);
    }
};

struct pjg_results {
    HitStore store;
    pjg_stats stats{};
    int device = 0;
    // count-only query: store.hits/atoms/warns are counts, nothing is kept
    bool count_only = false;
    const pjg_structures *structures = nullptr;  // the set the query searched
};

namespace {

// Device-to-host copy of result arrays into caller memory.  Small copies
// are plain cudaMemcpy.  Large ones are split into equal byte ranges, one
// per host thread: each thread first touches every page of its range of the
// caller's arrays (freshly allocated arrays are not yet mapped, and taking
// those page faults is what limits such a copy; measured on a GB300 host,
// 2.25 GB into untouched pages 81 ms, into touched ones 12 ms), then copies
// its range with cudaMemcpy straight into them.

struct CopySeg {
    void *dst;
    const void *src;
    size_t bytes;
};

// bytes [lo, hi) of the concatenation of `segs`, by one thread
cudaError_t copy_range(const std::vector<CopySeg> &segs, size_t lo, size_t hi, int device) {
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return e;
    size_t base = 0;
    for (const CopySeg &sg : segs) {
        const size_t a = std::max(lo, base), b = std::min(hi, base + sg.bytes);
        if (a < b) {
            volatile char *d = (volatile char *)sg.dst + (a - base);
            for (size_t x = 0; x < b - a; x += 4096) d[x] = 0;
            d[b - a - 1] = 0;
        }
        base += sg.bytes;
    }
    base = 0;
    for (const CopySeg &sg : segs) {
        const size_t a = std::max(lo, base), b = std::min(hi, base + sg.bytes);
        if (a < b) {
            e = cudaMemcpy((char *)sg.dst + (a - base), (const char *)sg.src + (a - base), b - a,
                           cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) return e;
        }
        base += sg.bytes;
    }
    return cudaSuccess;
}

cudaError_t copy_out_all(const std::vector<CopySeg> &segs_in) {
    std::vector<CopySeg> segs;
    size_t total = 0;
    for (const CopySeg &sg : segs_in)
        if (sg.dst && sg.bytes) {
            segs.push_back(sg);
            total += sg.bytes;
        }
    if (total == 0) return cudaSuccess;
    int device = 0;
    cudaGetDevice(&device);
    unsigned hw = std::thread::hardware_concurrency();
    // one thread per MiB, up to 16 (or the host's cores)
    int threads = (int)std::min<size_t>(std::min<unsigned>(hw ? hw : 1, 16u), total >> 20);
    if (threads <= 1) {
        for (const CopySeg &sg : segs) {
            cudaError_t e = cudaMemcpy(sg.dst, sg.src, sg.bytes, cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) return e;
        }
        return cudaSuccess;
    }
    const size_t slice = ((total + threads - 1) / threads + 4095) & ~size_t(4095);
    std::vector<cudaError_t> errs(threads, cudaSuccess);
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; t++) {
        const size_t lo = std::min(total, (size_t)t * slice), hi = std::min(total, lo + slice);
        pool.emplace_back([&, t, lo, hi] { errs[t] = copy_range(segs, lo, hi, device); });
    }
    for (auto &th : pool) th.join();
    for (cudaError_t e : errs)
        if (e != cudaSuccess) return e;
    return cudaSuccess;
}

cudaError_t copy_out(void *dst, const void *src, size_t bytes) { return copy_out_all({{dst, src, bytes}}); }

}  // namespace

extern "C" {

const char *pjg_last_error(void) { return g_error.c_str(); }

pjg_status pjg_init(int32_t device) {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0)
        return fail(PJG_ERR_NO_DEVICE, "no CUDA device: %s", e == cudaSuccess ? "count is 0" : cudaGetErrorString(e));
    if (device < 0 || device >= n) return fail(PJG_ERR_INVALID, "device %d out of range (%d devices)", device, n);
    e = cudaSetDevice(device);
    if (e != cudaSuccess) return fail(PJG_ERR_CUDA, "cudaSetDevice: %s", cudaGetErrorString(e));
    return PJG_OK;
}

// ---------------------------------------------------------------------------
// Templates

pjg_status pjg_templates_create(const pjg_template_set *set, pjg_templates **out) {
    pjg_status status = PJG_OK;
    if (!set || !out) return fail(PJG_ERR_INVALID, "null argument");
    if (set->n_templates < 0) return fail(PJG_ERR_INVALID, "negative template count");
    int T = set->n_templates;
    if (T > 0 && (!set->atom_offset)) return fail(PJG_ERR_INVALID, "null atom_offset");
    int A = T > 0 ? set->atom_offset[T] : 0;
    if (A > 0 && (!set->code || !set->res_seq || !set->chain || !set->xyz || !set->dist_weight ||
                  !set->name_offset || !set->resname_offset))
        return fail(PJG_ERR_INVALID, "null template atom array");
    pjg_templates *h = new pjg_templates;
    cudaGetDevice(&h->device);
    h->T = T;
    h->A = A;
    h->atom_begin.assign(set->atom_offset, set->atom_offset + T + 1);
    if (T == 0) h->atom_begin = {0};
    std::vector<int32_t> sig(A), key(A);
    std::vector<double> pos(3 * (size_t)A), weight(A);
    // signatures
    // signature ids by the bytes of (code, name count, names, residue names)
    std::unordered_map<std::string, int> sig_ids;
    sig_ids.reserve((size_t)A);
    std::vector<uint32_t> names, res, keyv;
    std::string keys;
    std::vector<int32_t> s_code, s_rule, s_main, s_nb{0}, s_rb{0}, s_pb{0};
    std::vector<uint32_t> s_names, s_res, s_pres, s_pname;
    for (int t = 0; t < T; t++) {
        int a0 = set->atom_offset[t], a1 = set->atom_offset[t + 1];
        if (a1 < a0) {
            delete h;
            return fail(PJG_ERR_INVALID, "template %d: decreasing atom offsets", t);
        }
        if (a1 - a0 > MAX_TEMPLATE_ATOMS) {
            delete h;
            return fail(PJG_ERR_INVALID, "template %d has %d atoms; at most %d are supported", t, a1 - a0,
                        MAX_TEMPLATE_ATOMS);
        }
        if (a1 - a0 > 32) h->large.push_back(t);
        h->nmax = std::max(h->nmax, a1 - a0);
    }
    for (int a = 0; a < A; a++) {
        int code = set->code[a];
        bool valid = (code >= -1 && code <= 8) || (code >= 100 && code <= 107);
        if (!valid) {
            delete h;
            return fail(PJG_ERR_INVALID, "template atom %d: invalid match mode %d", a, code);
        }
        names.clear();
        res.clear();
        for (int q = set->name_offset[a]; q < set->name_offset[a + 1]; q++) names.push_back(pack_upper(set->names + 4 * q));
        for (int q = set->resname_offset[a]; q < set->resname_offset[a + 1]; q++) {
            uint32_t r = pack_upper(set->resnames + 4 * q);
            if (std::find(res.begin(), res.end(), r) == res.end()) res.push_back(r);
        }
        keyv.clear();
        keyv.push_back((uint32_t)code);
        keyv.push_back((uint32_t)names.size());
        keyv.insert(keyv.end(), names.begin(), names.end());
        keyv.insert(keyv.end(), res.begin(), res.end());
        keys.assign(reinterpret_cast<const char *>(keyv.data()), keyv.size() * sizeof(uint32_t));
        auto it = sig_ids.find(keys);
        int id;
        if (it == sig_ids.end()) {
            id = (int)s_code.size();
            sig_ids.emplace(keys, id);
            int mode = code >= 100 ? code - 100 : code;
            int rule = mode == -1 ? RULE_ANY : mode == 1 ? RULE_NAME_OR_PARTNER : mode == 2 ? RULE_NAME_OR_MAINCHAIN
                     : mode == 3 ? RULE_ELEMENT : RULE_NAME;
            s_code.push_back(code);
            s_rule.push_back(rule);
            int mc = 0;
            for (uint32_t nm : names)
                if (nm == pack_lit("_CA_") || nm == pack_lit("_N__") || nm == pack_lit("_O__")) mc = 1;
            s_main.push_back(mc);
            s_names.insert(s_names.end(), names.begin(), names.end());
            s_nb.push_back((int32_t)s_names.size());
            s_res.insert(s_res.end(), res.begin(), res.end());
            s_rb.push_back((int32_t)s_res.size());
            if (rule == RULE_NAME_OR_PARTNER) {
                for (uint32_t nm : names)
                    for (const PartnerDef &p : PARTNER_TABLE) {
                        if (nm == pack_lit(p.a)) {
                            s_pres.push_back(res_lit(p.res));
                            s_pname.push_back(pack_lit(p.b));
                        }
                        if (nm == pack_lit(p.b)) {
                            s_pres.push_back(res_lit(p.res));
                            s_pname.push_back(pack_lit(p.a));
                        }
                    }
            }
            s_pb.push_back((int32_t)s_pres.size());
        } else {
            id = it->second;
        }
        sig[a] = id;
        key[a] = make_key(set->res_seq[a], set->chain[2 * a + 1]);
        for (int d = 0; d < 3; d++) pos[3 * (size_t)a + d] = set->xyz[3 * (size_t)a + d];
        weight[a] = set->dist_weight[a];
    }
    h->G = (int32_t)s_code.size();
    // distance matrices (TessAtom_distance, patches/TessAtom.c.patch:229-244;
    // Template.__init__, src/pyjess/_jess.pyx:1894-1901)
    std::vector<double> dist;
    h->param_begin.push_back(0);
    for (int t = 0; t < T; t++) {
        int a0 = set->atom_offset[t], n = set->atom_offset[t + 1] - a0;
        size_t base = dist.size();
        dist.resize(base + (size_t)n * n, 0.0);
        for (int i = 0; i < n; i++)
            for (int j = i + 1; j < n; j++) {
                double acc = 0.0;
                for (int d = 0; d < 3; d++) {
                    double tmp = pos[3 * (size_t)(a0 + i) + d] - pos[3 * (size_t)(a0 + j) + d];
                    acc += tmp * tmp;
                }
                acc = std::sqrt(acc);
                dist[base + (size_t)i * n + j] = acc;
                dist[base + (size_t)j * n + i] = acc;
            }
        h->param_begin.push_back((int32_t)dist.size());
    }
    if (dist.size() > (size_t)INT32_MAX) {
        delete h;
        return fail(PJG_ERR_INVALID, "templates too large: %zu distance-matrix entries (at most %d)", dist.size(),
                    INT32_MAX);
    }
    h->n_params = (int64_t)dist.size();
    if (set->dim) h->dim.assign(set->dim, set->dim + T);
    {
        cudaError_t e = cudaSuccess;
        if (e == cudaSuccess) e = upload(&h->d_atom_begin, h->atom_begin);
        if (e == cudaSuccess) e = upload(&h->d_sig, sig);
        if (e == cudaSuccess) e = upload(&h->d_key, key);
        if (e == cudaSuccess) e = upload(&h->d_param_begin, h->param_begin);
        if (e == cudaSuccess) e = upload(&h->d_pos, pos);
        if (e == cudaSuccess) e = upload(&h->d_weight, weight);
        if (e == cudaSuccess) e = upload(&h->d_dist, dist);
        if (e == cudaSuccess) e = upload(&h->d_code, s_code);
        if (e == cudaSuccess) e = upload(&h->d_rule, s_rule);
        if (e == cudaSuccess) e = upload(&h->d_mainchain, s_main);
        if (e == cudaSuccess) e = upload(&h->d_name_begin, s_nb);
        if (e == cudaSuccess) e = upload(&h->d_names, s_names);
        if (e == cudaSuccess) e = upload(&h->d_res_begin, s_rb);
        if (e == cudaSuccess) e = upload(&h->d_resnames, s_res);
        if (e == cudaSuccess) e = upload(&h->d_partner_begin, s_pb);
        if (e == cudaSuccess) e = upload(&h->d_partner_res, s_pres);
        if (e == cudaSuccess) e = upload(&h->d_partner_name, s_pname);
        if (e == cudaSuccess && !h->large.empty()) e = upload(&h->d_large, h->large);
        if (e != cudaSuccess) {
            status = fail(e == cudaErrorMemoryAllocation ? PJG_ERR_OOM : PJG_ERR_CUDA, "template upload: %s",
                          cudaGetErrorString(e));
            pjg_templates_destroy(h);
            return status;
        }
    }
    *out = h;
    return PJG_OK;
}

void pjg_templates_destroy(pjg_templates *h) {
    if (!h) return;
    void *ptrs[] = {h->d_atom_begin, h->d_sig, h->d_key, h->d_param_begin, h->d_pos, h->d_weight, h->d_dist,
                    h->d_code, h->d_rule, h->d_mainchain, h->d_name_begin, h->d_names, h->d_res_begin,
                    h->d_resnames, h->d_partner_begin, h->d_partner_res, h->d_partner_name, h->d_large};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    delete h;
}

// ---------------------------------------------------------------------------
// Structures

pjg_status pjg_structures_create(const pjg_structure_set *set, pjg_structures **out) {
    if (!set || !out) return fail(PJG_ERR_INVALID, "null argument");
    if (set->n_structures < 0) return fail(PJG_ERR_INVALID, "negative structure count");
    int S = set->n_structures;
    if (S > 0 && !set->atom_offset) return fail(PJG_ERR_INVALID, "null atom_offset");
    int64_t N = S > 0 ? set->atom_offset[S] : 0;
    if (N > 0 && (!set->xyz || !set->name || !set->resname || !set->chain || !set->res_seq || !set->serial))
        return fail(PJG_ERR_INVALID, "null structure atom array");
    pjg_structures *h = new pjg_structures;
    cudaGetDevice(&h->device);
    h->S = S;
    h->N = N;
    std::vector<int64_t> base(std::max(S, 0));
    std::vector<int32_t> count(std::max(S, 0));
    HostArray<float4> xyz32((size_t)N);
    HostArray<uint32_t> name((size_t)N), resname((size_t)N);
    HostArray<int32_t> sorted((size_t)N);
    HostArray<uint8_t> name_id((size_t)N);
    HostArray<int32_t> nh_pos((size_t)N);
    std::vector<int32_t> bucket_begin{0}, bucket_lo, bucket_hi;
    std::vector<uint32_t> bucket_name;
    for (int s = 0; s < S; s++) {
        int64_t b0 = set->atom_offset[s], b1 = set->atom_offset[s + 1];
        if (b1 < b0) {
            delete h;
            return fail(PJG_ERR_INVALID, "structure %d: decreasing atom offsets", s);
        }
        if (b1 - b0 > INT32_MAX / 2) {
            delete h;
            return fail(PJG_ERR_INVALID, "structure %d too large", s);
        }
        base[s] = b0;
        count[s] = (int)(b1 - b0);
        h->max_atoms = std::max(h->max_atoms, count[s]);
    }
    // per structure, on host threads: centroid-relative FP32 coordinates
    // with the residue key, packed names, and the ResIndex order (stable by
    // residue name, then serial) with its residue-name buckets
    struct Buckets {
        std::vector<uint32_t> name;
        std::vector<int32_t> lo, hi;
        std::vector<uint32_t> hname;  // distinct atom names of each bucket, sorted
        std::vector<int32_t> hcount, hbegin{0};
        std::vector<int32_t> hoff;    // start of each distinct name's atoms in nh_pos (structure-local)
        double radius = 0.0;
        int64_t bad = -1;  // first atom with a non-finite coordinate
    };
    std::vector<Buckets> bk(std::max(S, 0));
    auto prepare = [&](int s) {
        const int64_t b0 = base[s];
        const int n = count[s];
        Buckets &B = bk[s];
        for (int i = 0; i < n && B.bad < 0; i++)
            for (int d = 0; d < 3; d++)
                if (!std::isfinite(set->xyz[3 * (b0 + i) + d])) B.bad = i;
        if (B.bad >= 0) return;
        double c[3] = {0, 0, 0};
        for (int i = 0; i < n; i++)
            for (int d = 0; d < 3; d++) c[d] += set->xyz[3 * (b0 + i) + d];
        if (n > 0)
            for (int d = 0; d < 3; d++) c[d] /= (double)n;
        for (int i = 0; i < n; i++) {
            int64_t a = b0 + i;
            double dx = set->xyz[3 * a] - c[0], dy = set->xyz[3 * a + 1] - c[1], dz = set->xyz[3 * a + 2] - c[2];
            double r = std::sqrt(dx * dx + dy * dy + dz * dz);
            if (r > B.radius) B.radius = r;
            int32_t k = make_key(set->res_seq[a], set->chain[2 * a + 1]);
            float kf;
            std::memcpy(&kf, &k, 4);
            xyz32[a] = make_float4((float)dx, (float)dy, (float)dz, kf);
            name[a] = pack_upper(set->name + 4 * a);
            resname[a] = pack_upper(set->resname + 4 * a);
        }
        // ResIndex: stable order by (residue name, serial) -- a counting
        // sort by residue name (in byte order of the upper-cased name), then
        // a stable sort by serial of each bucket not already in serial order
        std::vector<int32_t> idx(n);
        {
            std::vector<std::pair<uint32_t, int32_t>> kinds;  // big-endian name, count
            std::vector<int32_t> kind(n);
            for (int i = 0; i < n; i++) {
                const uint8_t *r = set->resname + 4 * (b0 + i);
                const uint32_t k = ((uint32_t)up(r[0]) << 24) | ((uint32_t)up(r[1]) << 16) |
                                   ((uint32_t)up(r[2]) << 8) | up(r[3]);
                int q = 0;
                while (q < (int)kinds.size() && kinds[q].first != k) q++;
                if (q == (int)kinds.size()) kinds.push_back({k, 0});
                kinds[q].second++;
                kind[i] = q;
            }
            std::vector<int> by(kinds.size());
            std::iota(by.begin(), by.end(), 0);
            std::sort(by.begin(), by.end(), [&](int x, int y) { return kinds[x].first < kinds[y].first; });
            std::vector<int32_t> start(kinds.size());
            int acc = 0;
            for (int q : by) {
                start[q] = acc;
                acc += kinds[q].second;
            }
            std::vector<int32_t> fill = start;
            for (int i = 0; i < n; i++) idx[fill[kind[i]]++] = i;
            const int32_t *ser = set->serial + b0;
            for (size_t q = 0; q < kinds.size(); q++) {
                int32_t *lo = idx.data() + start[q], *hi = lo + kinds[q].second;
                bool ordered = true;
                for (int32_t *x = lo; x + 1 < hi && ordered; x++) ordered = ser[x[0]] <= ser[x[1]];
                if (!ordered) std::stable_sort(lo, hi, [&](int x, int y) { return ser[x] < ser[y]; });
            }
        }
        for (int i = 0; i < n; i++) {
            sorted[b0 + i] = idx[i];
            uint32_t rn = resname[b0 + idx[i]];
            if (i == 0 || rn != B.name.back()) {
                if (i > 0) B.hi.push_back(i);
                B.name.push_back(rn);
                B.lo.push_back(i);
            }
        }
        if (n > 0) B.hi.push_back(n);
        // per bucket: its distinct atom names and their counts
        std::vector<uint32_t> nm;
        for (size_t k = 0; k < B.name.size(); k++) {
            nm.clear();
            for (int i = B.lo[k]; i < B.hi[k]; i++) nm.push_back(name[b0 + idx[i]]);
            std::sort(nm.begin(), nm.end());
            const size_t h0 = B.hname.size();
            for (size_t i = 0; i < nm.size(); i++) {
                if (i == 0 || nm[i] != nm[i - 1]) {
                    B.hname.push_back(nm[i]);
                    B.hcount.push_back(0);
                }
                B.hcount.back()++;
            }
            B.hbegin.push_back((int32_t)B.hname.size());
            // the bucket's atoms grouped by name (groups in name order, each
            // in ResIndex order), from the bucket's first position
            std::vector<int32_t> fill(B.hname.size() - h0);
            for (size_t j = 0, acc = (size_t)B.lo[k]; j < fill.size(); j++) {
                fill[j] = (int32_t)acc;
                B.hoff.push_back((int32_t)acc);
                acc += (size_t)B.hcount[h0 + j];
            }
            for (int i = B.lo[k]; i < B.hi[k]; i++) {
                const int a = idx[i];
                const size_t id = std::lower_bound(B.hname.begin() + h0, B.hname.end(), name[b0 + a]) -
                                  (B.hname.begin() + h0);
                name_id[b0 + a] = (uint8_t)std::min<size_t>(id, 255);
                nh_pos[b0 + fill[id]++] = a;
            }
        }
    };
    {
        const int nthreads = (int)std::max<unsigned>(1, std::min<unsigned>(32, std::thread::hardware_concurrency()));
        std::atomic<int> next{0};
        auto worker = [&]() {
            for (int s; (s = next.fetch_add(1)) < S;) prepare(s);
        };
        std::vector<std::thread> pool;
        for (int i = 1; i < std::min(nthreads, S); i++) pool.emplace_back(worker);
        worker();
        for (auto &th : pool) th.join();
    }
    for (int s = 0; s < S; s++)
        if (bk[s].bad >= 0) {
            delete h;
            return fail(PJG_ERR_INVALID, "structure %d atom %lld: non-finite coordinate", s, (long long)bk[s].bad);
        }
    std::vector<int32_t> nh_begin{0}, nh_count, nh_off;
    std::vector<uint32_t> nh_name;
    for (int s = 0; s < S; s++) {
        const Buckets &B = bk[s];
        for (size_t k = 0; k + 1 < B.hbegin.size(); k++) nh_begin.push_back((int32_t)nh_name.size() + B.hbegin[k + 1]);
        nh_name.insert(nh_name.end(), B.hname.begin(), B.hname.end());
        nh_count.insert(nh_count.end(), B.hcount.begin(), B.hcount.end());
        nh_off.insert(nh_off.end(), B.hoff.begin(), B.hoff.end());
    }
    for (int s = 0; s < S; s++) {
        const Buckets &B = bk[s];
        h->max_radius = std::max(h->max_radius, B.radius);
        bucket_name.insert(bucket_name.end(), B.name.begin(), B.name.end());
        bucket_lo.insert(bucket_lo.end(), B.lo.begin(), B.lo.end());
        bucket_hi.insert(bucket_hi.end(), B.hi.begin(), B.hi.end());
        bucket_begin.push_back((int32_t)bucket_name.size());
    }
    h->atom_base = base;
    cudaError_t e = cudaMalloc((void **)&h->d_xyz64, std::max<size_t>(3 * (size_t)N, 1) * sizeof(double));
    if (e == cudaSuccess && N > 0)
        e = cudaMemcpy(h->d_xyz64, set->xyz, 3 * (size_t)N * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = upload(&h->d_atom_base, base);
    if (e == cudaSuccess) e = upload(&h->d_atom_count, count);
    if (e == cudaSuccess) e = upload(&h->d_xyz32, xyz32.p.get(), (size_t)N);
    if (e == cudaSuccess) e = upload(&h->d_name, name.p.get(), (size_t)N);
    if (e == cudaSuccess) e = upload(&h->d_resname, resname.p.get(), (size_t)N);
    if (e == cudaSuccess) e = upload(&h->d_sorted, sorted.p.get(), (size_t)N);
    if (e == cudaSuccess) e = upload(&h->d_bucket_begin, bucket_begin);
    if (e == cudaSuccess) e = upload(&h->d_bucket_name, bucket_name);
    if (e == cudaSuccess) e = upload(&h->d_bucket_lo, bucket_lo);
    if (e == cudaSuccess) e = upload(&h->d_bucket_hi, bucket_hi);
    if (e == cudaSuccess) e = upload(&h->d_nh_begin, nh_begin);
    if (e == cudaSuccess) e = upload(&h->d_nh_name, nh_name);
    if (e == cudaSuccess) e = upload(&h->d_nh_count, nh_count);
    if (e == cudaSuccess) e = upload(&h->d_name_id, name_id.p.get(), (size_t)N);
    if (e == cudaSuccess) e = upload(&h->d_nh_off, nh_off);
    if (e == cudaSuccess) e = upload(&h->d_nh_pos, nh_pos.p.get(), (size_t)N);
    if (e == cudaSuccess) {
        // axis ranks of every atom (the leaf-order sorted-axis path)
        const size_t n3 = 3 * (size_t)std::max<int64_t>(N, 1);
        unsigned long long *tile_key = nullptr;
        uint16_t *tile_idx = nullptr;
        e = cudaMalloc((void **)&h->d_lrank, n3 * sizeof(uint32_t));
        if (e == cudaSuccess) e = cudaMalloc((void **)&h->d_urank, n3 * sizeof(uint32_t));
        if (e == cudaSuccess) e = cudaMalloc((void **)&tile_key, n3 * sizeof(unsigned long long));
        if (e == cudaSuccess) e = cudaMalloc((void **)&tile_idx, n3 * sizeof(uint16_t));
        if (e == cudaSuccess) {
            launch_axis_ranks(0, S, h->d_atom_base, h->d_atom_count, h->d_xyz64, N, tile_key, tile_idx, h->d_lrank,
                              h->d_urank);
            e = cudaGetLastError();
            if (e == cudaSuccess) e = cudaDeviceSynchronize();
        }
        if (tile_key) cudaFree(tile_key);
        if (tile_idx) cudaFree(tile_idx);
    }
    if (e != cudaSuccess) {
        pjg_status st = fail(e == cudaErrorMemoryAllocation ? PJG_ERR_OOM : PJG_ERR_CUDA, "structure upload: %s",
                             cudaGetErrorString(e));
        pjg_structures_destroy(h);
        return st;
    }
    *out = h;
    return PJG_OK;
}

void pjg_structures_destroy(pjg_structures *h) {
    if (!h) return;
    void *ptrs[] = {h->d_atom_base, h->d_atom_count, h->d_xyz64, h->d_xyz32, h->d_name, h->d_resname,
                    h->d_sorted, h->d_bucket_begin, h->d_bucket_name, h->d_bucket_lo, h->d_bucket_hi,
                    h->d_lrank, h->d_urank, h->d_nh_begin, h->d_nh_name, h->d_nh_count, h->d_name_id,
                    h->d_nh_off, h->d_nh_pos};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    delete h;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Query

namespace {

__global__ void k_struct_totals(int32_t S, int32_t G, const int32_t *count, int64_t *totals) {
    int lane = threadIdx.x & 31;
    int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t s = warp; s < S; s += nw) {
        int64_t acc = 0;
        for (int g = lane; g < G; g += 32) acc += count[s * G + g];
        for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) totals[s] = acc;
    }
}

int sm_count() {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

// exclusive scan in[0..n) -> out[0..n), recursive over tile sums
// kernels launched by scan_exclusive on this thread (query statistics)
thread_local int t_scan_launches = 0;

template <typename T>
cudaError_t scan_exclusive(const T *in, int64_t n, int64_t *out, std::vector<DBuf<int64_t>> &tmp,
                           cudaStream_t st, int depth = 0) {
    if (n <= 0) return cudaSuccess;
    t_scan_launches += n > SCAN_TILE_ITEMS ? 2 : 1;
    const int TILE = SCAN_TILE_ITEMS;
    int64_t tiles = (n + TILE - 1) / TILE;
    if ((int)tmp.size() < 2 * (depth + 1)) tmp.resize(2 * (depth + 1));
    cudaError_t e = dalloc(tmp[2 * depth], (size_t)tiles, st);
    if (e != cudaSuccess) return e;
    e = dalloc(tmp[2 * depth + 1], (size_t)tiles, st);
    if (e != cudaSuccess) return e;
    int64_t *sums = tmp[2 * depth].p, *soff = tmp[2 * depth + 1].p;
    if constexpr (sizeof(T) == 4) launch_scan_tiles_i32(st, in, n, out, sums);
    else launch_scan_tiles_i64(st, in, n, out, sums);
    if (tiles > 1) {
        e = scan_exclusive<int64_t>(sums, tiles, soff, tmp, st, depth + 1);
        if (e != cudaSuccess) return e;
        launch_scan_add(st, out, n, soff);
    }
    return cudaGetLastError();
}

#if PJG_SEARCH_PROF
// Profile builds: append the query's search profile as one JSON line to the
// file named by PJG_PROF_OUT (nothing when unset).
void write_search_profile(const unsigned long long *d_prof, cudaStream_t st, const pjg_stats &stats) {
    static const char *names[SP_NUM] = {
        "pairs", "empty", "cyc_pair", "cyc_setup", "cyc_seed", "cyc_block", "cyc_prod", "cyc_emit",
        "loop_iters", "block_visits", "block_visits_l0", "chain_full", "chain_sibling", "g0_iters",
        "blocks_tested", "blocks_hit", "leaves_inbox", "batches", "batch_lanes", "child_block",
        "prod_batches", "prod_batches_l0", "prod_lanes", "child_prod", "fp64", "rows", "cyc_chain", "cyc_batch", "cyc_ctrl", "cyc_susp",
        "tail_ns", "pair_max_cyc"};
    unsigned long long h[SP_NUM] = {};
    if (cudaMemcpyAsync(h, d_prof, sizeof h, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return;
    const char *path = getenv("PJG_PROF_OUT");
    if (!path || !*path) return;
    FILE *f = fopen(path, "a");
    if (!f) return;
    fprintf(f, "{\"ms_expansion\": %.3f, \"partials\": %lld, \"search_rounds\": %d", stats.ms_expansion,
            (long long)stats.partials, stats.search_rounds);
    for (int i = 0; i < SP_NUM; i++) fprintf(f, ", \"%s\": %llu", names[i], h[i]);
    static const char *lnames[LP_CLASS] = {"lists", "entries", "handed", "cyc_list", "cyc_load", "cyc_sort",
                                           "cyc_count", "cyc_seg", "cyc_write", "sort_nodes", "sort_words",
                                           "count_pairs"};
    unsigned long long lh[LP_NUM] = {};
    leaf_profile_read(lh, st);
    cudaStreamSynchronize(st);
    fprintf(f, ", \"leaf_order\": {");
    for (int i = 0; i < LP_CLASS; i++) fprintf(f, "%s\"%s\": %llu", i ? ", " : "", lnames[i], lh[i]);
    const char *cls[3] = {"class_lists", "class_entries", "class_cycles"};
    for (int k = 0; k < 3; k++) {
        fprintf(f, ", \"%s\": [", cls[k]);
        for (int c = 0; c < 7; c++) fprintf(f, "%s%llu", c ? ", " : "", lh[LP_CLASS + 7 * k + c]);
        fprintf(f, "]");
    }
    fprintf(f, "}}\n");
    fclose(f);
}
#endif

}  // namespace

// ---------------------------------------------------------------------------
// Execution tuning (process-wide, read at the start of each query)

namespace {
std::mutex g_tuning_mutex;
constexpr pjg_tuning TUNING_DEFAULTS = {4, 64, 4096, 1, LEAF_RANK_MAX, -1};
pjg_tuning g_tuning = TUNING_DEFAULTS;

pjg_tuning current_tuning() {
    std::lock_guard<std::mutex> g(g_tuning_mutex);
    return g_tuning;
}
}  // namespace

extern "C" pjg_status pjg_set_tuning(const pjg_tuning *t) {
    pjg_tuning d = TUNING_DEFAULTS;
    if (t) {
        if (t->leaf_levels < -1 || t->leaf_levels > 64) return fail(PJG_ERR_INVALID, "leaf_levels %d", t->leaf_levels);
        if (t->block_min < 0 || t->block_min > 65535) return fail(PJG_ERR_INVALID, "block_min %d", t->block_min);
        if (t->tile_cap != 0 && (t->tile_cap < 32 || t->tile_cap > 16384))
            return fail(PJG_ERR_INVALID, "tile_cap %d", t->tile_cap);
        if (t->pair_grain < 0 || t->pair_grain > 64) return fail(PJG_ERR_INVALID, "pair_grain %d", t->pair_grain);
        if (t->leaf_rank_max < 0 || t->leaf_rank_max > LEAF_FAST_MAX)
            return fail(PJG_ERR_INVALID, "leaf_rank_max %d", t->leaf_rank_max);
        if (t->leaf_reach < -1 || t->leaf_reach > 64) return fail(PJG_ERR_INVALID, "leaf_reach %d", t->leaf_reach);
        if (t->leaf_levels) d.leaf_levels = t->leaf_levels;
        if (t->block_min) d.block_min = t->block_min;
        if (t->tile_cap) d.tile_cap = t->tile_cap;
        if (t->pair_grain) d.pair_grain = t->pair_grain;
        if (t->leaf_rank_max) d.leaf_rank_max = t->leaf_rank_max;
        if (t->leaf_reach) d.leaf_reach = t->leaf_reach;
    }
    std::lock_guard<std::mutex> g(g_tuning_mutex);
    g_tuning = d;
    return PJG_OK;
}

extern "C" pjg_status pjg_get_tuning(pjg_tuning *t) {
    if (!t) return fail(PJG_ERR_INVALID, "null argument");
    *t = current_tuning();
    return PJG_OK;
}

extern "C" pjg_status pjg_device_name(char *buf, int32_t len) {
    if (!buf || len <= 0) return fail(PJG_ERR_INVALID, "null or empty buffer");
    int dev = 0;
    cudaDeviceProp prop;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaGetDeviceProperties(&prop, dev);
    if (e != cudaSuccess) {
        buf[0] = 0;
        return fail(PJG_ERR_NO_DEVICE, "no CUDA device: %s", cudaGetErrorString(e));
    }
    snprintf(buf, (size_t)len, "%s", prop.name);
    return PJG_OK;
}

extern "C" pjg_status pjg_query(const pjg_templates *tp, const pjg_structures *sp, const pjg_query_params *P,
                                pjg_results **out) {
    pjg_status status = PJG_OK;
    if (!tp || !sp || !P || !out) return fail(PJG_ERR_INVALID, "null argument");
    if (P->ignore_chain < 0 || P->ignore_chain > 2) return fail(PJG_ERR_INVALID, "invalid ignore_chain %d", P->ignore_chain);
    if (P->max_candidates < -1) return fail(PJG_ERR_INVALID, "invalid max_candidates %d", P->max_candidates);
    if (P->mode < 0 || P->mode > 2) return fail(PJG_ERR_INVALID, "invalid mode %d", P->mode);
    if (P->count_only < 0 || P->count_only > 1) return fail(PJG_ERR_INVALID, "invalid count_only %d", P->count_only);
    if (!std::isfinite(P->distance_cutoff) || !std::isfinite(P->max_dynamic_distance))
        return fail(PJG_ERR_INVALID, "non-finite distance parameters");

    pjg_results *res = new pjg_results;
    cudaGetDevice(&res->device);
    res->count_only = P->count_only != 0;
    res->structures = sp;
    const int T = tp->T, S = sp->S, G = tp->G;
    const bool fp32 = P->mode == PJG_MODE_BATCHED_FP32;
    cudaStream_t st = nullptr;
    cudaEvent_t ev[8] = {};
    DBuf<AnnulusParam> d_params;
    DBuf<int32_t> d_count, d_scanned, d_cand_atom, d_leaf_atom, d_pair_counter;
    DBuf<int64_t> d_offset, d_totals, d_boff;
    DBuf<int32_t> d_nblk;
    DBuf<int64_t> d_exact_list, d_sorted_list;
    DBuf<unsigned long long> d_exact_count, d_sorted_count;
    DBuf<float4> d_blk_lo, d_blk_hi;
    DBuf<float4> d_leaf_xyz, d_leaf_xyz2;
    DBuf<int32_t> d_leaf_atom2;
    DBuf<int64_t> d_leaf_off;
    DBuf<unsigned long long> d_leaf_used;
    DBuf<unsigned long long> d_counters, d_ccount, d_rtotals;
    DBuf<int32_t> d_c_pair, d_c_atoms, d_pair_rows, d_cnt_q;
    DBuf<int64_t> d_c_ord, d_off_q;
    // lists ordered on demand: per-list state, requested lists, suspended pairs
    DBuf<int32_t> d_lstate;
    DBuf<int64_t> d_work;
    DBuf<unsigned long long> d_nwork, d_nsusp;
    // lists filled on demand
    DBuf<int32_t> d_fill_state;
    DBuf<int64_t> d_fill_work;
    DBuf<unsigned long long> d_nfill;
    DBuf<Suspended> d_susp_a, d_susp_b;
    DBuf<unsigned char> d_pool_a, d_pool_b;
    // costliest pairs first: cost buckets, heavy flags and list, histogram
    DBuf<uint8_t> d_pcost, d_hflag;
    DBuf<int32_t> d_heavy;
    DBuf<unsigned long long> d_hbins;
    DBuf<unsigned long long> d_pool_used;
    int64_t pool_cap = 0;
    // requested lists sharing one leaf order (table and worklists)
    DBuf<unsigned long long> d_ls_key, d_ls_n;
    DBuf<int32_t> d_ls_rep, d_ls_slot;
    DBuf<int64_t> d_ls_rep_work, d_ls_dup, d_ls_left;
    DBuf<uint8_t> d_ls_ok;
    DBuf<double> d_c_rmsd;
    DBuf<unsigned long long> d_prof;  // search profile (profile builds)
    // per complete row, in reference order
    DBuf<double> d_r_rmsd, d_r_rot, d_r_cen;
    DBuf<int32_t> d_r_nan, d_r_hit, d_r_warn, d_r_hatoms;
    DBuf<int64_t> d_r_src, d_r_hidx, d_r_widx, d_r_aidx;
    std::vector<DBuf<int64_t>> scan_tmp;
    int64_t passing = 0;
    const int stride = std::max(tp->nmax, 1);
    unsigned long long counters[C_NUM] = {};
    float ms = 0.f;
    double ms_cand = 0, ms_exp = 0, ms_sup = 0, ms_total = 0, ms_search = 0;
    int launches = 0, chunks = 0, search_rounds = 0, row_splits = 0;
    t_scan_launches = 0;
    int64_t suspensions = 0;
    // levels whose lists are put in kd leaf order before the search (deeper
    // lists when a pair's frontier first reaches them): the tuning's
    // leaf_levels, or PJG_LEAF_LEVELS when set; a negative value orders
    // every list up front.  The plain per-structure path orders every list
    // up front: with one structure a chunk, the host round trip of each
    // extra search round costs more than the ordering it saves.
    const pjg_tuning tune = current_tuning();
    int demand_levels = P->mode == PJG_MODE_PLAIN_FP64 ? -1 : tune.leaf_levels;
    {
        const char *v = getenv("PJG_LEAF_LEVELS");
        if (v && *v && P->mode != PJG_MODE_PLAIN_FP64) demand_levels = atoi(v);
    }
    std::vector<int64_t> totals(S);

    if (T == 0 || S == 0) {
        *out = res;
        return PJG_OK;
    }
    {
        int dev = 0;
        cudaGetDevice(&dev);
        if (dev != tp->device || dev != sp->device) {
            delete res;
            return fail(PJG_ERR_INVALID, "templates, structures and the calling thread use different devices");
        }
    }
    {
        // keep the stream-ordered pool's memory mapped between queries (up
        // to half the device) instead of returning it at every sync: the
        // next query's chunk buffers then need no new mappings
        static std::mutex m;
        static bool done[256] = {};
        std::lock_guard<std::mutex> g(m);
        if (res->device >= 0 && res->device < 256 && !done[res->device]) {
            cudaMemPool_t pool;
            size_t fb = 0, tb = 0;
            if (cudaDeviceGetDefaultMemPool(&pool, res->device) == cudaSuccess && cudaMemGetInfo(&fb, &tb) == cudaSuccess) {
                uint64_t thr = tb / 2;
                cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
            }
            cudaGetLastError();
            done[res->device] = true;
        }
    }
    CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
#if PJG_SEARCH_PROF
    leaf_profile_reset(st);
#endif
    for (auto &e : ev) CUDA_TRY(cudaEventCreate(&e));
    CUDA_TRY(cudaEventRecord(ev[0], st));

    {
        // guard band: the requested width, widened if the FP32 rounding bound
        // of the largest structure needs more.  Coordinates are stored
        // relative to the structure's centroid, so each is within about
        // 2^-24 R of its FP64 value (R = largest distance from the centroid)
        // and the error of an FP32 squared distance d^2 is below
        // 2^-24 (10.4 R d + 4 d^2); a band g in distance covers a band of
        // about 2 b g in squared distance at radius b, so g must exceed
        // 2^-24 (5.2 R + 2 b), with b at most 2 R + 1 for any pair of atoms
        // (plus the tolerance) inside a structure.
        double g = P->guard_band > 0 ? P->guard_band : 1e-4;
        double bound = 2.0 * std::ldexp(1.0, -24) * (5.2 * sp->max_radius + 2.0 * (2.0 * sp->max_radius + 1.0));
        if (bound > g) g = bound;
        CUDA_TRY(dalloc(d_params, (size_t)std::max<int64_t>(tp->n_params, 1), st));
        launch_params(st, T, tp->d_atom_begin, tp->d_param_begin, tp->d_dist, tp->d_weight,
                      P->distance_cutoff, P->max_dynamic_distance, g, d_params.p);
        launches++;
        CUDA_TRY(cudaGetLastError());
    }
    CUDA_TRY(dalloc(d_counters, C_NUM, st));
    CUDA_TRY(cudaMemsetAsync(d_counters.p, 0, C_NUM * sizeof(unsigned long long), st));
    CUDA_TRY(dalloc(d_pair_counter, 1, st));
    CUDA_TRY(dalloc(d_ccount, 1, st));
    CUDA_TRY(dalloc(d_rtotals, 4, st));

    {
        // pass 1: list lengths for every (structure, signature)
        int64_t W = (int64_t)S * G;
        CUDA_TRY(dalloc(d_count, (size_t)W, st));
        CUDA_TRY(dalloc(d_scanned, (size_t)W, st));
        CUDA_TRY(dalloc(d_totals, (size_t)S, st));
        ChunkView cv{S, sp->d_atom_base, sp->d_atom_count, sp->d_xyz64, sp->d_xyz32, sp->d_name, sp->d_resname,
                     sp->d_sorted, sp->d_bucket_begin, sp->d_bucket_name, sp->d_bucket_lo, sp->d_bucket_hi,
                     sp->N, sp->d_lrank, sp->d_urank, sp->d_nh_begin, sp->d_nh_name, sp->d_nh_count,
                     sp->d_name_id, sp->d_nh_off, sp->d_nh_pos};
        SigView sv{G, tp->d_code, tp->d_rule, tp->d_mainchain, tp->d_name_begin, tp->d_names, tp->d_res_begin,
                   tp->d_resnames, tp->d_partner_begin, tp->d_partner_res, tp->d_partner_name};
        int blocks = (int)std::min<int64_t>((W + 7) / 8, (int64_t)sm_count() * 32);
        launch_candidates(st, std::max(blocks, 1), false, cv, sv, d_count.p, d_scanned.p, nullptr, nullptr);
        k_struct_totals<<<std::max(1, std::min(S, sm_count() * 8)), 256, 0, st>>>(S, G, d_count.p, d_totals.p);
        launches += 2;
        CUDA_TRY(cudaGetLastError());
        CUDA_TRY(cudaMemcpyAsync(totals.data(), d_totals.p, sizeof(int64_t) * S, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
    }

    {
        // chunks of structures under an entry budget.  A candidate entry
        // costs at most ENTRY_BYTES: its atom in candidate order (4), block
        // boxes (32 B a block of CULL_BLK leaves), per-list arrays (~1) and,
        // once its list is put in leaf order, its atom and FP32 point in
        // leaf order (20; allocated as lists are requested).  The budget
        // takes 60% of the free device memory (counting memory the
        // stream-ordered pool holds unused) at that worst case, at least 48M
        // entries, which leaves room for growing the leaf arrays (old and new
        // copies live at once while they grow).  Fewer, larger chunks leave
        // fewer kernel tails and search rounds.  PJG_ENTRY_BUDGET overrides
        // it.
        constexpr double ENTRY_BYTES = 25.0 + 32.0 / CULL_BLK;
        int64_t ENTRY_BUDGET = 48ll << 20;
        {
            size_t free_b = 0, total_b = 0;
            if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess) {
                cudaMemPool_t pool;
                if (cudaDeviceGetDefaultMemPool(&pool, res->device) == cudaSuccess) {
                    uint64_t reserved = 0, used = 0;
                    if (cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &reserved) == cudaSuccess &&
                        cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used) == cudaSuccess &&
                        reserved > used)
                        free_b += (size_t)(reserved - used);
                }
                cudaGetLastError();
                ENTRY_BUDGET = std::max<int64_t>(ENTRY_BUDGET, (int64_t)((double)free_b * 0.6 / ENTRY_BYTES));
            }
            const char *v = getenv("PJG_ENTRY_BUDGET");
            if (v && atoll(v) > 0) ENTRY_BUDGET = atoll(v);
        }
        const int max_chunk = P->mode == PJG_MODE_PLAIN_FP64 ? 1 : 4096;
        // structures a chunk may take; halved when a chunk's complete rows
        // outgrow the memory of the per-row stages (see below), then sized
        // from the rows a structure of the last chunk produced
        int chunk_cap = max_chunk;
        const bool cut_inline = !P->best_match && P->max_candidates >= 0;
        // device bytes a complete row takes: its record in the row buffers
        // (grown with a quarter of headroom) and the per-row stages after the
        // search (superposition, automaton, compaction and the hits they may
        // append)
        const double row_buf_bytes = 12.0 + 4.0 * stride + (cut_inline ? 8.0 : 0.0);
        const double row_stage_bytes = 360.0 + 4.0 * stride;
        // memory a chunk's rows may use: free device memory, memory the
        // stream-ordered pool holds unused, and the row buffers and per-row
        // arrays of the previous chunk (reused)
        auto row_memory = [&]() -> double {
            double a = 0.0;
            size_t free_b = 0, total_b = 0;
            if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess) a = (double)free_b;
            cudaMemPool_t pool;
            if (cudaDeviceGetDefaultMemPool(&pool, res->device) == cudaSuccess) {
                uint64_t reserved = 0, used = 0;
                if (cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &reserved) == cudaSuccess &&
                    cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used) == cudaSuccess &&
                    reserved > used)
                    a += (double)(reserved - used);
            }
            cudaGetLastError();
            a += (double)(d_c_pair.n * 4 + d_c_ord.n * 8 + d_c_atoms.n * 4 + d_c_rmsd.n * 8);
            a += (double)(d_r_rmsd.n * 8 + d_r_rot.n * 8 + d_r_cen.n * 8 + d_r_nan.n * 4 + d_r_src.n * 8 +
                          d_r_hit.n * 4 + d_r_warn.n * 4 + d_r_hatoms.n * 4 + d_r_hidx.n * 8 + d_r_widx.n * 8 +
                          d_r_aidx.n * 8);
            return a;
        };
        // rows a chunk may produce (PJG_ROW_BUDGET sets it)
        auto row_budget = [&]() -> int64_t {
            const char *v = getenv("PJG_ROW_BUDGET");
            if (v && atoll(v) > 0) return atoll(v);
            return (int64_t)(0.7 * row_memory() / (row_buf_bytes * 1.25 + row_stage_bytes));
        };
        // best_match with max_candidates: a pair stops after max_candidates
        // + 2 complete rows, so a structure yields at most T times that; the
        // chunks are sized from this bound before any search (no chunk then
        // needs a split)
        int bound_cap = max_chunk;
        if (P->best_match && P->max_candidates >= 0 && max_chunk > 1) {
            const double per = (double)T * ((double)P->max_candidates + 2.0);
            bound_cap = (int)std::max(1.0, std::min((double)max_chunk, (double)row_budget() / per));
            chunk_cap = bound_cap;
        }
        int s0 = 0;
        int64_t c_cap = 1 << 20;
        CUDA_TRY(dalloc(d_c_pair, c_cap, st));
        CUDA_TRY(dalloc(d_c_ord, c_cap, st));
        CUDA_TRY(dalloc(d_c_atoms, (size_t)c_cap * stride, st));
        if (cut_inline) CUDA_TRY(dalloc(d_c_rmsd, c_cap, st));
        while (s0 < S) {
            int s1 = s0;
            int64_t entries = 0;
            while (s1 < S && (s1 == s0 || (entries + totals[s1] <= ENTRY_BUDGET && s1 - s0 < chunk_cap))) {
                entries += totals[s1];
                s1++;
            }
            chunks++;
            const double ms_search_chunk0 = ms_search;
            // host statistics and device counters before this chunk (restored
            // if it is redone on fewer structures)
            const int search_rounds0 = search_rounds;
            const int64_t suspensions0 = suspensions;
            unsigned long long chunk_snap[C_NUM];
            CUDA_TRY(cudaMemcpyAsync(chunk_snap, d_counters.p, sizeof chunk_snap, cudaMemcpyDeviceToHost, st));
            CUDA_TRY(cudaStreamSynchronize(st));
            const int Sc = s1 - s0;
            const int64_t Wc = (int64_t)Sc * G;
            ChunkView cv{Sc, sp->d_atom_base + s0, sp->d_atom_count + s0, sp->d_xyz64, sp->d_xyz32, sp->d_name,
                         sp->d_resname, sp->d_sorted, sp->d_bucket_begin + s0, sp->d_bucket_name, sp->d_bucket_lo,
                         sp->d_bucket_hi, sp->N, sp->d_lrank, sp->d_urank, sp->d_nh_begin, sp->d_nh_name,
                         sp->d_nh_count, sp->d_name_id, sp->d_nh_off, sp->d_nh_pos};
            SigView sv{G, tp->d_code, tp->d_rule, tp->d_mainchain, tp->d_name_begin, tp->d_names, tp->d_res_begin,
                       tp->d_resnames, tp->d_partner_begin, tp->d_partner_res, tp->d_partner_name};
            int32_t *cnt_c = d_count.p + (int64_t)s0 * G;
            int32_t *scn_c = d_scanned.p + (int64_t)s0 * G;
            CUDA_TRY(dalloc(d_offset, (size_t)Wc, st));
            CUDA_TRY(cudaEventRecord(ev[1], st));
            CUDA_TRY(scan_exclusive(cnt_c, Wc, d_offset.p, scan_tmp, st));
            // culling blocks of CULL_BLK leaves: counts, offsets, total (one
            // small sync)
            int64_t nblocks = 0;
            CUDA_TRY(dalloc(d_nblk, (size_t)Wc, st));
            CUDA_TRY(dalloc(d_boff, (size_t)Wc, st));
            launch_block_counts(st, Wc, cnt_c, d_nblk.p);
            CUDA_TRY(scan_exclusive(d_nblk.p, Wc, d_boff.p, scan_tmp, st));
            {
                int64_t lastoff = 0;
                int32_t lastn = 0;
                CUDA_TRY(cudaMemcpyAsync(&lastoff, d_boff.p + Wc - 1, 8, cudaMemcpyDeviceToHost, st));
                CUDA_TRY(cudaMemcpyAsync(&lastn, d_nblk.p + Wc - 1, 4, cudaMemcpyDeviceToHost, st));
                CUDA_TRY(cudaStreamSynchronize(st));
                nblocks = lastoff + lastn;
            }
            CUDA_TRY(dalloc(d_blk_lo, (size_t)std::max<int64_t>(nblocks, 1), st));
            CUDA_TRY(dalloc(d_blk_hi, (size_t)std::max<int64_t>(nblocks, 1), st));
            CUDA_TRY(dalloc(d_cand_atom, (size_t)entries, st));
            // leaf-order arrays: every entry when every list is ordered up
            // front, else half of them to start with (grown on demand;
            // PJG_LEAF_CAPACITY sets the starting size)
            {
                int64_t cap0 = demand_levels < 0 ? entries : std::max<int64_t>(entries / 2, 1 << 20);
                const char *v = getenv("PJG_LEAF_CAPACITY");
                if (demand_levels >= 0 && v && atoll(v) > 0) {
                    cap0 = atoll(v);
                    dfree(d_leaf_atom, st);
                    dfree(d_leaf_xyz, st);
                }
                CUDA_TRY(dalloc(d_leaf_atom, (size_t)cap0, st));
            }
            CUDA_TRY(dalloc(d_leaf_xyz, d_leaf_atom.n, st));
            int64_t leaf_filled = 0;  // leaf entries of the lists ordered so far
            const int fill_blocks = std::max(1, (int)std::min<int64_t>((Wc + 7) / 8, (int64_t)sm_count() * 32));
            {
                // every list is filled here when every list is put in leaf
                // order up front; otherwise only the lists a search reads:
                // the level-0 list of each pair that can run (queued by
                // k_demand_levels) and each list put in leaf order (filled
                // just before it is ordered)
                if (demand_levels < 0) {
                    launch_candidates(st, fill_blocks, true, cv, sv, nullptr, nullptr, d_offset.p, d_cand_atom.p);
                    launches++;
                }
                CUDA_TRY(dalloc(d_exact_list, (size_t)Wc, st));
                CUDA_TRY(dalloc(d_exact_count, 1, st));
                CUDA_TRY(dalloc(d_sorted_list, (size_t)LEAF_LISTS * (size_t)Wc, st));
                CUDA_TRY(dalloc(d_sorted_count, LEAF_LISTS, st));
                launches++;  // block counts
                CUDA_TRY(cudaGetLastError());
            }
            TemplateView tv{T, tp->nmax, tp->d_atom_begin, tp->d_sig, tp->d_pos, tp->d_key, tp->d_param_begin,
                            d_params.p};
            if (demand_levels >= 0) CUDA_TRY(dalloc(d_leaf_off, (size_t)Wc, st));
            const int64_t *leaf_off = demand_levels < 0 ? d_offset.p : d_leaf_off.p;
            CandView cd{G, cnt_c, d_offset.p, d_cand_atom.p, leaf_off, d_leaf_atom.p, d_leaf_xyz.p,
                        d_boff.p, d_blk_lo.p, d_blk_hi.p};
            const int64_t n_pairs = (int64_t)Sc * T;
            // kd leaf order: up front for the lists of the first
            // `demand_levels` levels of every pair that can run, later (between
            // search rounds) for each deeper list a pair's frontier reaches;
            // a negative value orders every list of the chunk up front
            LeafDemand dm{};
            const int leaf_blocks =
                std::max(1, (int)std::min<int64_t>((Wc + LEAF_WARPS - 1) / LEAF_WARPS, (int64_t)sm_count() * 32));
            // room in the leaf arrays for `need` entries (the lists ordered so
            // far keep their places)
            auto ensure_leaf = [&](int64_t need) -> cudaError_t {
                if (need <= (int64_t)d_leaf_atom.n) return cudaSuccess;
                const size_t cap2 = (size_t)std::max<int64_t>(need + need / 4, (int64_t)d_leaf_atom.n * 3 / 2);
                cudaError_t e = dalloc(d_leaf_atom2, cap2, st);
                if (e == cudaSuccess) e = dalloc(d_leaf_xyz2, cap2, st);
                if (e != cudaSuccess) return e;
                if (leaf_filled > 0) {
                    e = cudaMemcpyAsync(d_leaf_atom2.p, d_leaf_atom.p, (size_t)leaf_filled * sizeof(int32_t),
                                        cudaMemcpyDeviceToDevice, st);
                    if (e == cudaSuccess)
                        e = cudaMemcpyAsync(d_leaf_xyz2.p, d_leaf_xyz.p, (size_t)leaf_filled * sizeof(float4),
                                            cudaMemcpyDeviceToDevice, st);
                    if (e != cudaSuccess) return e;
                }
                std::swap(d_leaf_atom, d_leaf_atom2);
                std::swap(d_leaf_xyz, d_leaf_xyz2);
                dfree(d_leaf_atom2, st);
                dfree(d_leaf_xyz2, st);
                cd.leaf_atom = d_leaf_atom.p;
                cd.leaf_xyz = d_leaf_xyz.p;
                return cudaSuccess;
            };
            // lists of the same atoms share one leaf order (demand mode only:
            // there the leaf offsets are a separate, writable array)
            ListShare ls{};
            bool share_on = false;
            auto order_requested = [&]() -> cudaError_t {
                if (dm.fill_state) {
                    // the requested lists not filled yet
                    launch_candidates(st, fill_blocks, true, cv, sv, nullptr, nullptr, d_offset.p, d_cand_atom.p,
                                      dm.work, dm.n_work, dm.fill_state, true);
                    launches++;
                }
                if (share_on) {
                    // key every requested list, order one list per key, point
                    // the others at its leaves, order those whose atoms differ
                    const cudaError_t e0 = cudaMemsetAsync(ls.n, 0, 3 * sizeof(unsigned long long), st);
                    if (e0 != cudaSuccess) return e0;
                    launch_list_keys(st, sm_count() * 16, G, cnt_c, d_offset.p, d_cand_atom.p, dm.work, dm.n_work,
                                     ls, d_counters.p);
                    launch_list_reps(st, sm_count() * 16, dm.work, dm.n_work, ls);
                    launch_leaf_order(st, leaf_blocks, cv, G, cnt_c, d_offset.p, d_boff.p, d_cand_atom.p, leaf_off,
                                      d_leaf_atom.p, d_leaf_xyz.p, d_blk_lo.p, d_blk_hi.p, d_sorted_list.p,
                                      d_sorted_count.p, Wc, d_exact_list.p, d_exact_count.p, d_counters.p,
                                      ls.rep_work, ls.n, tune.leaf_rank_max, ls.part_ok, 0);
                    launch_list_share(st, sm_count() * 8, cv, G, cnt_c, d_offset.p, d_cand_atom.p, d_leaf_off.p,
                                      d_boff.p, ls, d_counters.p);
                    launch_leaf_order(st, leaf_blocks, cv, G, cnt_c, d_offset.p, d_boff.p, d_cand_atom.p, leaf_off,
                                      d_leaf_atom.p, d_leaf_xyz.p, d_blk_lo.p, d_blk_hi.p, d_sorted_list.p,
                                      d_sorted_count.p, Wc, d_exact_list.p, d_exact_count.p, d_counters.p,
                                      ls.left_work, ls.n + 2, tune.leaf_rank_max, ls.part_ok, 0);
                    launches += 2 * LEAF_ORDER_LAUNCHES + 3;
                } else {
                    launch_leaf_order(st, leaf_blocks, cv, G, cnt_c, d_offset.p, d_boff.p, d_cand_atom.p, leaf_off,
                                      d_leaf_atom.p, d_leaf_xyz.p, d_blk_lo.p, d_blk_hi.p, d_sorted_list.p,
                                      d_sorted_count.p, Wc, d_exact_list.p, d_exact_count.p, d_counters.p, dm.work,
                                      dm.n_work, tune.leaf_rank_max);
                    launches += LEAF_ORDER_LAUNCHES;
                }
                if (dm.state) {
                    launch_mark_ordered(st, sm_count() * 4, dm);
                    launches++;
                }
                return cudaGetLastError();
            };
            if (demand_levels < 0) {
                CUDA_TRY(order_requested());
            } else {
                CUDA_TRY(dalloc(d_lstate, (size_t)Wc, st));
                CUDA_TRY(dalloc(d_work, (size_t)Wc, st));
                CUDA_TRY(dalloc(d_nwork, 1, st));
                CUDA_TRY(dalloc(d_nsusp, 1, st));
                CUDA_TRY(dalloc(d_susp_a, (size_t)n_pairs, st));
                CUDA_TRY(dalloc(d_susp_b, (size_t)n_pairs, st));
                if (pool_cap == 0) {
                    // saved search states of suspended pairs, one pool per
                    // round in turn: a sixteenth of the free memory each,
                    // 64 MiB to 4 GiB (a pair that finds its pool full is
                    // rerun from its start instead)
                    size_t free_b = 0, total_b = 0;
                    int64_t cap = 64ll << 20;
                    if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess)
                        cap = std::max<int64_t>(cap, std::min<int64_t>(4ll << 30, (int64_t)(free_b / 16)));
                    const char *v = getenv("PJG_STATE_POOL");
                    if (v && atoll(v) >= 0) cap = atoll(v);
                    pool_cap = std::max<int64_t>(cap, 16);
                    CUDA_TRY(dalloc(d_pool_a, (size_t)pool_cap, st));
                    CUDA_TRY(dalloc(d_pool_b, (size_t)pool_cap, st));
                    CUDA_TRY(dalloc(d_pool_used, 1, st));
                }
                dm.pool_used = d_pool_used.p;
                dm.pool_cap = pool_cap;
                CUDA_TRY(cudaMemsetAsync(d_lstate.p, 0, (size_t)Wc * sizeof(int32_t), st));
                CUDA_TRY(cudaMemsetAsync(d_nwork.p, 0, sizeof(unsigned long long), st));
                dm.state = d_lstate.p;
                dm.work = d_work.p;
                dm.n_work = d_nwork.p;
                dm.n_suspended = d_nsusp.p;
                CUDA_TRY(dalloc(d_leaf_used, 1, st));
                CUDA_TRY(cudaMemsetAsync(d_leaf_used.p, 0, sizeof(unsigned long long), st));
                dm.leaf_offset = d_leaf_off.p;
                dm.leaf_used = d_leaf_used.p;
                CUDA_TRY(dalloc(d_fill_state, (size_t)Wc, st));
                CUDA_TRY(dalloc(d_fill_work, (size_t)Wc, st));
                CUDA_TRY(dalloc(d_nfill, 1, st));
                CUDA_TRY(cudaMemsetAsync(d_fill_state.p, 0, (size_t)Wc * sizeof(int32_t), st));
                CUDA_TRY(cudaMemsetAsync(d_nfill.p, 0, sizeof(unsigned long long), st));
                dm.fill_state = d_fill_state.p;
                dm.fill_work = d_fill_work.p;
                dm.n_fill = d_nfill.p;
                {
                    // the list-sharing table: twice the chunk's lists, a power
                    // of two (without the memory, every list is ordered)
                    int64_t cap = 1;
                    while (cap < 2 * Wc) cap <<= 1;
                    cudaError_t e = dalloc(d_ls_key, (size_t)cap, st);
                    if (e == cudaSuccess) e = dalloc(d_ls_rep, (size_t)cap, st);
                    if (e == cudaSuccess) e = dalloc(d_ls_slot, (size_t)Wc, st);
                    if (e == cudaSuccess) e = dalloc(d_ls_rep_work, (size_t)Wc, st);
                    if (e == cudaSuccess) e = dalloc(d_ls_dup, (size_t)Wc, st);
                    if (e == cudaSuccess) e = dalloc(d_ls_left, (size_t)Wc, st);
                    if (e == cudaSuccess) e = dalloc(d_ls_n, 3, st);
                    if (e == cudaSuccess) e = dalloc(d_ls_ok, (size_t)Wc, st);
                    if (e == cudaSuccess) e = cudaMemsetAsync(d_ls_key.p, 0, (size_t)cap * sizeof(unsigned long long), st);
                    if (e == cudaSuccess) e = cudaMemsetAsync(d_ls_rep.p, 0xFF, (size_t)cap * sizeof(int32_t), st);
                    if (e == cudaSuccess) e = cudaMemsetAsync(d_ls_ok.p, 0, (size_t)Wc, st);
                    // PJG_LIST_SHARING=0 orders every list itself
                    const char *v = getenv("PJG_LIST_SHARING");
                    share_on = e == cudaSuccess && !(v && v[0] == '0');
                    if (e != cudaSuccess) {
                        cudaGetLastError();
                        dfree(d_ls_key, st);
                        dfree(d_ls_rep, st);
                        dfree(d_ls_slot, st);
                        dfree(d_ls_rep_work, st);
                        dfree(d_ls_dup, st);
                        dfree(d_ls_left, st);
                        dfree(d_ls_ok, st);
                    }
                    ls.key = d_ls_key.p;
                    ls.rep = d_ls_rep.p;
                    ls.mask = cap - 1;
                    ls.slot = d_ls_slot.p;
                    ls.rep_work = d_ls_rep_work.p;
                    ls.dup_work = d_ls_dup.p;
                    ls.left_work = d_ls_left.p;
                    ls.n = d_ls_n.p;
                    ls.part_ok = d_ls_ok.p;
                }
                if (n_pairs > INT32_MAX) {
                    status = fail(PJG_ERR_CAPACITY, "too many pairs in one chunk");
                    goto done;
                }
                // the costliest pairs are searched first (a pair can take
                // milliseconds; started last, it alone would run on while the
                // other warps idle): the level demand estimates each pair's
                // cost, and the pairs of the top cost buckets, at most two
                // (PJG_HEAVY_PER_WARP) per resident search warp, are taken
                // before the others
                const char *hw = getenv("PJG_HEAVY_PER_WARP");
                const int64_t per_warp = hw && atoi(hw) > 0 ? atoi(hw) : 2;
                const int64_t heavy_target = per_warp * 2 * sm_count() * SEARCH_WARPS;
                const char *hf = getenv("PJG_HEAVY_FIRST");
                const bool heavy_on = (int64_t)n_pairs >= 8 * heavy_target &&
                                      (int64_t)n_pairs <= (int64_t)INT32_MAX - heavy_target &&
                                      !(hf && atoi(hf) == 0);
                dm.pair_cost = nullptr;
                dm.heavy = nullptr;
                if (heavy_on) {
                    CUDA_TRY(dalloc(d_pcost, (size_t)n_pairs, st));
                    CUDA_TRY(dalloc(d_hflag, (size_t)n_pairs, st));
                    CUDA_TRY(dalloc(d_heavy, (size_t)heavy_target, st));
                    CUDA_TRY(dalloc(d_hbins, 66, st));
                    CUDA_TRY(cudaMemsetAsync(d_hbins.p, 0, 66 * sizeof(unsigned long long), st));
                    dm.pair_cost = d_pcost.p;
                }
                launch_demand_levels(st, sm_count() * 16, tv, cd, (int32_t)n_pairs, demand_levels, P->reorder, dm);
                if (heavy_on) {
                    launch_heavy_pairs(st, (int32_t)n_pairs, d_pcost.p, d_hbins.p, heavy_target, d_hflag.p,
                                       d_heavy.p);
                    dm.heavy = d_heavy.p;
                    dm.n_heavy = d_hbins.p + 64;
                    dm.heavy_flag = d_hflag.p;
                    launches += 2;
                }
                // the level-0 lists the pairs read in candidate order
                launch_candidates(st, fill_blocks, true, cv, sv, nullptr, nullptr, d_offset.p, d_cand_atom.p,
                                  dm.fill_work, dm.n_fill, nullptr, false);
                launches += 2;
                unsigned long long used = 0;
                CUDA_TRY(cudaMemcpyAsync(&used, d_leaf_used.p, sizeof used, cudaMemcpyDeviceToHost, st));
                CUDA_TRY(cudaStreamSynchronize(st));
                CUDA_TRY(ensure_leaf((int64_t)used));
                CUDA_TRY(order_requested());
                leaf_filled = (int64_t)used;
            }
            CUDA_TRY(cudaEventRecord(ev[2], st));
            SearchArgs sa;
            sa.n_pairs = Sc * T;
            if (n_pairs > INT32_MAX) {
                status = fail(PJG_ERR_CAPACITY, "too many pairs in one chunk");
                goto done;
            }
            sa.ignore_chain = P->ignore_chain;
            sa.reorder = P->reorder;
            sa.best_match = P->best_match;
            sa.max_candidates = P->max_candidates;
            {
                // shared memory per warp: pair state + tiles of >= 64
                // entries for every level but the last (k_search takes
                // templates of up to 32 atoms)
                int levels = std::max(1, std::min(tp->nmax, 32) - 1);
                size_t entry = sp->max_atoms > 65535 ? 8 : 4;
                size_t need = search_state_bytes() + entry * 64 * (size_t)levels;
                sa.warp_smem = (int)((std::max<size_t>(need, search_state_bytes() + 5376) + 15) & ~size_t(15));
            }
            sa.cut_inline = cut_inline ? 1 : 0;
            sa.rmsd_threshold = P->rmsd_threshold;
            sa.prof = nullptr;
            sa.block_min = tune.block_min;
            sa.tile_cap = tune.tile_cap;
            sa.pair_grain = tune.pair_grain;
            sa.leaf_reach = tune.leaf_reach;
#if PJG_SEARCH_PROF
            if (!d_prof.p) {
                CUDA_TRY(dalloc(d_prof, SP_NUM, st));
                CUDA_TRY(cudaMemsetAsync(d_prof.p, 0, SP_NUM * sizeof(unsigned long long), st));
            }
            sa.prof = d_prof.p;
#endif
            {
                const char *b = getenv("PJG_KERNEL_BUDGET_S");
                double sec = b ? atof(b) : 120.0;
                if (!(sec > 0)) sec = 120.0;
                sa.budget_ns = (uint64_t)(sec * 1e9);
            }
            bool wide = sp->max_atoms > 65535;
            // counters before this chunk's search, restored if it must rerun
            unsigned long long snap[C_NUM];
            CUDA_TRY(cudaMemcpyAsync(snap, d_counters.p, sizeof snap, cudaMemcpyDeviceToHost, st));
            CUDA_TRY(cudaStreamSynchronize(st));
            CUDA_TRY(dalloc(d_pair_rows, (size_t)n_pairs, st));
            // room before the first attempt (a rerun of the search costs a
            // whole chunk): two complete rows a pair, or, with best_match
            // and max_candidates, the most a pair can produce (max_candidates
            // + 2) when the row budget takes that
            int64_t want_rows = 2 * n_pairs;
            if (P->best_match && P->max_candidates >= 0) {
                const int64_t bound = n_pairs * ((int64_t)P->max_candidates + 2);
                const int64_t budget = row_budget();
                if (bound <= budget) {
                    want_rows = std::max(want_rows, bound);
                } else if (Sc > 1) {
                    // with the chunk's own lists in memory its bound no
                    // longer fits: take fewer structures before searching
                    chunk_cap = std::max(1, (int)((double)Sc * (double)budget / (double)bound));
                    bound_cap = std::min(bound_cap, chunk_cap);
                    chunks--;
                    row_splits++;
                    CUDA_TRY(cudaMemcpyAsync(d_counters.p, chunk_snap, sizeof chunk_snap, cudaMemcpyHostToDevice,
                                             st));
                    continue;
                }
            }
            if (c_cap < want_rows) {
                c_cap = want_rows;
                CUDA_TRY(dalloc(d_c_pair, c_cap, st));
                CUDA_TRY(dalloc(d_c_ord, c_cap, st));
                CUDA_TRY(dalloc(d_c_atoms, (size_t)c_cap * stride, st));
                if (cut_inline) CUDA_TRY(dalloc(d_c_rmsd, c_cap, st));
            }
            // set when the chunk's complete rows cannot be held: the chunk is
            // redone on half its structures
            bool split = false;
            for (int attempt = 0; attempt < 8; attempt++) {
                CUDA_TRY(cudaMemsetAsync(d_ccount.p, 0, sizeof(unsigned long long), st));
                CUDA_TRY(cudaMemsetAsync(d_pair_rows.p, 0, (size_t)n_pairs * sizeof(int32_t), st));
                CompleteRows cr{d_ccount.p, c_cap, stride, d_c_pair.p, d_c_ord.p, d_c_atoms.p,
                                cut_inline ? d_c_rmsd.p : nullptr, d_pair_rows.p};
                int grid = sm_count() * 8;
                unsigned long long nc = 0;
                // search rounds: every pair, then the pairs suspended at a
                // list that had no leaf order (ordered in between), until
                // no pair is suspended
                dm.resume = nullptr;
                dm.n_resume = 0;
                dm.pool_in = nullptr;
                Suspended *next_out = d_susp_a.p, *spare = d_susp_b.p;
                unsigned char *pool_next = d_pool_a.p, *pool_spare = d_pool_b.p;
                for (int round = 0;; round++) {
                    CUDA_TRY(cudaMemsetAsync(d_pair_counter.p, 0, sizeof(int32_t), st));
                    if (dm.state) {
                        dm.suspended = next_out;
                        dm.pool_out = pool_next;
                        CUDA_TRY(cudaMemsetAsync(d_nwork.p, 0, sizeof(unsigned long long), st));
                        CUDA_TRY(cudaMemsetAsync(d_nsusp.p, 0, sizeof(unsigned long long), st));
                        CUDA_TRY(cudaMemsetAsync(d_pool_used.p, 0, sizeof(unsigned long long), st));
                    }
                    CUDA_TRY(cudaEventRecord(ev[6], st));
                    CUDA_TRY(launch_search(st, grid, wide, fp32, cv, tv, cd, sa, d_pair_counter.p, scn_c, cr,
                                           d_counters.p, dm));
                    launches++;
                    if (round == 0 && !tp->large.empty()) {
                        // pairs of templates over 32 atoms (every list of
                        // theirs was ordered before this round)
                        CUDA_TRY(cudaMemsetAsync(d_pair_counter.p, 0, sizeof(int32_t), st));
                        CUDA_TRY(launch_search_large(st, cv, tv, cd, sa, tp->d_large, (int32_t)tp->large.size(),
                                                     d_pair_counter.p, scn_c, cr, d_counters.p, dm.state));
                        launches++;
                    }
                    CUDA_TRY(cudaEventRecord(ev[7], st));
                    CUDA_TRY(cudaGetLastError());
                    unsigned long long ns = 0, used = 0;
                    CUDA_TRY(cudaMemcpyAsync(&nc, d_ccount.p, sizeof nc, cudaMemcpyDeviceToHost, st));
                    if (dm.state) {
                        CUDA_TRY(cudaMemcpyAsync(&ns, d_nsusp.p, sizeof ns, cudaMemcpyDeviceToHost, st));
                        CUDA_TRY(cudaMemcpyAsync(&used, d_leaf_used.p, sizeof used, cudaMemcpyDeviceToHost, st));
                    }
                    CUDA_TRY(cudaStreamSynchronize(st));
                    {
                        float m = 0.f;
                        cudaEventElapsedTime(&m, ev[6], ev[7]);
                        ms_search += m;
                    }
                    search_rounds++;
                    if (ns == 0) break;
                    if (round > 80) {
                        status = fail(PJG_ERR_CAPACITY, "leaf order on demand did not converge");
                        goto done;
                    }
                    suspensions += (int64_t)ns;
                    // the lists the suspended pairs reached, then those pairs
                    CUDA_TRY(ensure_leaf((int64_t)used));
                    CUDA_TRY(order_requested());
                    leaf_filled = (int64_t)used;
                    dm.resume = next_out;
                    dm.n_resume = (int32_t)ns;
                    dm.pool_in = pool_next;
                    std::swap(next_out, spare);
                    std::swap(pool_next, pool_spare);
                }
                if ((int64_t)nc <= c_cap) break;
                // the row buffer was too small: grow and run the chunk again
                // (the search counters of the failed attempt are rolled back;
                // lists ordered meanwhile stay ordered).  Rows beyond the
                // chunk's row budget, or a growth that fails, split the chunk
                // instead (down to one structure).
                if (Sc > 1 && (int64_t)nc > row_budget()) {
                    split = true;
                    break;
                }
                c_cap = (int64_t)nc + nc / 4 + 1024;
                {
                    cudaError_t eg = dalloc(d_c_pair, c_cap, st);
                    if (eg == cudaSuccess) eg = dalloc(d_c_ord, c_cap, st);
                    if (eg == cudaSuccess) eg = dalloc(d_c_atoms, (size_t)c_cap * stride, st);
                    if (eg == cudaSuccess && cut_inline) eg = dalloc(d_c_rmsd, c_cap, st);
                    if (eg == cudaErrorMemoryAllocation && Sc > 1) {
                        cudaGetLastError();
                        c_cap = std::min<int64_t>({(int64_t)d_c_pair.n, (int64_t)d_c_ord.n,
                                                   (int64_t)(d_c_atoms.n / stride)});
                        if (cut_inline) c_cap = std::min<int64_t>(c_cap, (int64_t)d_c_rmsd.n);
                        split = true;
                        break;
                    }
                    CUDA_TRY(eg);
                }
                {
                    unsigned long long cur[C_NUM];
                    CUDA_TRY(cudaMemcpyAsync(cur, d_counters.p, sizeof cur, cudaMemcpyDeviceToHost, st));
                    CUDA_TRY(cudaStreamSynchronize(st));
                    for (int c : {C_LEAF_EXACT, C_LEAF_SORTED, C_LEAF_REPLAY, C_LEAF_LISTS, C_LEAF_ENTRIES, C_LEAF_SHARED, C_ERROR})
                        snap[c] = cur[c];
                }
                CUDA_TRY(cudaMemcpyAsync(d_counters.p, snap, sizeof snap, cudaMemcpyHostToDevice, st));
            }
            CUDA_TRY(cudaEventRecord(ev[3], st));
            {
                // superposition of every complete row into its slot in
                // reference order, Query.__next__ per pair, compaction of
                // the hits and warnings into this chunk's segment
                unsigned long long nc = 0;
                CUDA_TRY(cudaMemcpyAsync(&nc, d_ccount.p, sizeof nc, cudaMemcpyDeviceToHost, st));
                CUDA_TRY(cudaStreamSynchronize(st));
                const int64_t rows = (int64_t)nc;
                // the per-row stages below hold ~360 + 4 * stride bytes a
                // complete row: when the chunk's rows need more than 70% of
                // the memory they may use, or the row buffers could not hold
                // them, the chunk is redone on half its structures
                const int64_t budget_now = row_budget();
                if (Sc > 1 && (split || rows > budget_now)) {
                    // at most half the structures, fewer when the rows seen
                    // say so (rows scale with the structures of a chunk)
                    const double fit = 0.8 * (double)Sc * (double)budget_now / (double)std::max<int64_t>(rows, 1);
                    chunk_cap = std::max(1, std::min(Sc / 2, (int)fit));
                    chunks--;
                    row_splits++;
                    search_rounds = search_rounds0;
                    suspensions = suspensions0;
                    ms_search = ms_search_chunk0;
                    CUDA_TRY(cudaMemcpyAsync(d_counters.p, chunk_snap, sizeof chunk_snap, cudaMemcpyHostToDevice,
                                             st));
                    continue;
                }
                CompleteRows cr{d_ccount.p, c_cap, stride, d_c_pair.p, d_c_ord.p, d_c_atoms.p,
                                cut_inline ? d_c_rmsd.p : nullptr, d_pair_rows.p};
                if (rows > 0) {
                    CUDA_TRY(dalloc(d_cnt_q, (size_t)n_pairs, st));
                    CUDA_TRY(dalloc(d_off_q, (size_t)n_pairs, st));
                    launch_order_counts(st, n_pairs, T, d_pair_rows.p, d_cnt_q.p);
                    CUDA_TRY(scan_exclusive(d_cnt_q.p, n_pairs, d_off_q.p, scan_tmp, st));
                    CUDA_TRY(dalloc(d_r_rmsd, (size_t)rows, st));
                    CUDA_TRY(dalloc(d_r_rot, (size_t)rows * 9, st));
                    CUDA_TRY(dalloc(d_r_cen, (size_t)rows * 6, st));
                    CUDA_TRY(dalloc(d_r_nan, (size_t)rows, st));
                    CUDA_TRY(dalloc(d_r_src, (size_t)rows, st));
                    CUDA_TRY(dalloc(d_r_hit, (size_t)rows, st));
                    CUDA_TRY(dalloc(d_r_warn, (size_t)rows, st));
                    CUDA_TRY(dalloc(d_r_hatoms, (size_t)rows, st));
                    CUDA_TRY(dalloc(d_r_hidx, (size_t)rows, st));
                    CUDA_TRY(dalloc(d_r_widx, (size_t)rows, st));
                    CUDA_TRY(dalloc(d_r_aidx, (size_t)rows, st));
                    RowResults rr{d_off_q.p, T, d_r_rmsd.p, d_r_nan.p, d_r_rot.p, d_r_cen.p, d_r_src.p};
                    int blocks = (int)std::min<int64_t>((rows + 127) / 128, (int64_t)sm_count() * 24);
                    launch_superpose(st, blocks, cv, tv, cr, rr);
                    CUDA_TRY(cudaMemsetAsync(d_rtotals.p, 0, 4 * sizeof(unsigned long long), st));
                    launch_automaton(st, n_pairs, T, tp->d_atom_begin, d_cnt_q.p, d_off_q.p, rr, P->max_candidates,
                                     P->best_match, P->rmsd_threshold, d_r_hit.p, d_r_warn.p, d_r_hatoms.p,
                                     d_rtotals.p);
                    CUDA_TRY(scan_exclusive(d_r_hit.p, rows, d_r_hidx.p, scan_tmp, st));
                    CUDA_TRY(scan_exclusive(d_r_warn.p, rows, d_r_widx.p, scan_tmp, st));
                    CUDA_TRY(scan_exclusive(d_r_hatoms.p, rows, d_r_aidx.p, scan_tmp, st));
                    unsigned long long tot[4] = {};
                    CUDA_TRY(cudaMemcpyAsync(tot, d_rtotals.p, sizeof tot, cudaMemcpyDeviceToHost, st));
                    CUDA_TRY(cudaStreamSynchronize(st));
                    passing += (int64_t)tot[3];
                    if (P->count_only) {
                        // counts only: the hits and warnings are not kept
                        res->store.hits += (int64_t)tot[0];
                        res->store.atoms += (int64_t)tot[2];
                        res->store.warns += (int64_t)tot[1];
                    } else if (tot[0] + tot[1] > 0) {
                        HitStore &hs = res->store;
                        CUDA_TRY(hs.reserve((int64_t)tot[0], (int64_t)tot[2], (int64_t)tot[1], st));
                        launch_gather_hits(st, rows, T, s0, hs.atoms, tp->d_atom_begin, cr, rr, d_r_hit.p,
                                           d_r_warn.p, d_r_hidx.p, d_r_widx.p, d_r_aidx.p, P->best_match, hs.tail());
                        CUDA_TRY(cudaGetLastError());
                        hs.hits += (int64_t)tot[0];
                        hs.atoms += (int64_t)tot[2];
                        hs.warns += (int64_t)tot[1];
                    }
                    launches += 8;
                }
                CUDA_TRY(cudaEventRecord(ev[4], st));
                float m1 = 0, m2 = 0, m3 = 0;
                CUDA_TRY(cudaEventSynchronize(ev[4]));
                cudaEventElapsedTime(&m1, ev[1], ev[2]);
                cudaEventElapsedTime(&m2, ev[2], ev[3]);
                cudaEventElapsedTime(&m3, ev[3], ev[4]);
                // search launches count as expansion; the leaf order run
                // between search rounds counts with the candidate lists
                ms_cand += m1 + (m2 - (float)(ms_search - ms_search_chunk0));
                ms_exp += ms_search - ms_search_chunk0;
                ms_sup += m3;
                // next chunk: as many structures as the row budget takes at
                // this chunk's rows per structure (a dense chunk early in the
                // set does not keep every later chunk small)
                if (rows > 0 && max_chunk > 1) {
                    const double per = (double)rows / (double)Sc;
                    const double fit = 0.8 * (double)row_budget() / per;
                    chunk_cap = (int)std::max(1.0, std::min((double)max_chunk, fit));
                } else {
                    chunk_cap = max_chunk;
                }
                chunk_cap = std::max(chunk_cap, std::min(bound_cap, max_chunk));
            }
            s0 = s1;
        }
    }
    CUDA_TRY(cudaMemcpyAsync(counters, d_counters.p, sizeof counters, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaEventRecord(ev[5], st));
    CUDA_TRY(cudaStreamSynchronize(st));
    cudaEventElapsedTime(&ms, ev[0], ev[5]);
    ms_total = ms;
    if (counters[C_ERROR] == 3) {
        status = fail(PJG_ERR_TIMEOUT, "search kernel exceeded its time budget (PJG_KERNEL_BUDGET_S)");
        goto done;
    }
    if (counters[C_ERROR]) {
        const unsigned long long c = counters[C_ERROR];
        status = fail(PJG_ERR_CAPACITY, "kernel reported error %llu (%s)", c,
                      c == 2 ? "template too large for the frontier tile"
                      : c == 4 ? "leaf order: too many small subtrees" : c == 5 ? "leaf order: partition did not converge"
                      : c == 7 ? "a list of a template over 32 atoms had no kd leaf order"
                      : "leaf order: inconsistent node partition");
        goto done;
    }

    res->stats.pairs = (int64_t)counters[C_PAIRS];
    res->stats.candidate_entries = (int64_t)counters[C_CAND];
    res->stats.partials = (int64_t)counters[C_PARTIALS];
    res->stats.complete = (int64_t)counters[C_COMPLETE];
    res->stats.passing = passing;
    res->stats.hits = res->store.hits;
    res->stats.fp64_rechecks = (int64_t)counters[C_RECHECK];
    res->stats.leaf_exact = (int64_t)counters[C_LEAF_EXACT];
    res->stats.leaf_sorted = (int64_t)counters[C_LEAF_SORTED];
    res->stats.leaf_replays = (int64_t)counters[C_LEAF_REPLAY];
    res->stats.bytes_candidates = (int64_t)counters[C_BYTES_CAND];
    res->stats.bytes_expansion = (int64_t)counters[C_BYTES_EXP];
    // per hit: its atoms, rmsd, rotation and centroids
    res->stats.bytes_superposition = 4 * res->store.atoms + (8 + 72 + 48) * res->store.hits;
    res->stats.ms_candidates = ms_cand;
    res->stats.ms_expansion = ms_exp;
    res->stats.ms_superposition = ms_sup;
    res->stats.ms_total = ms_total;
    res->stats.launches = launches + t_scan_launches;
    res->stats.chunks = chunks;
    res->stats.leaf_lists = (int64_t)counters[C_LEAF_LISTS];
    res->stats.leaf_entries = (int64_t)counters[C_LEAF_ENTRIES];
    res->stats.suspensions = suspensions;
    res->stats.search_rounds = search_rounds;
    res->stats.row_splits = row_splits;
    res->stats.leaf_shared = (int64_t)counters[C_LEAF_SHARED];
#if PJG_SEARCH_PROF
    if (d_prof.p) write_search_profile(d_prof.p, st, res->stats);
#endif

done:
    if (st) {
        dfree(d_params, st); dfree(d_count, st); dfree(d_scanned, st); dfree(d_cand_atom, st);
        dfree(d_leaf_atom, st); dfree(d_pair_counter, st); dfree(d_offset, st); dfree(d_totals, st);
        dfree(d_leaf_xyz, st); dfree(d_leaf_atom2, st); dfree(d_leaf_xyz2, st); dfree(d_leaf_off, st);
        dfree(d_leaf_used, st); dfree(d_counters, st); dfree(d_ccount, st);
        dfree(d_rtotals, st); dfree(d_c_pair, st); dfree(d_c_atoms, st); dfree(d_pair_rows, st);
        dfree(d_cnt_q, st); dfree(d_c_ord, st); dfree(d_off_q, st); dfree(d_c_rmsd, st); dfree(d_boff, st);
        dfree(d_nblk, st); dfree(d_blk_lo, st); dfree(d_blk_hi, st); dfree(d_exact_list, st);
        dfree(d_exact_count, st); dfree(d_sorted_list, st); dfree(d_sorted_count, st);
        dfree(d_r_rmsd, st); dfree(d_r_rot, st); dfree(d_r_cen, st); dfree(d_r_nan, st); dfree(d_r_hit, st);
        dfree(d_r_warn, st); dfree(d_r_hatoms, st); dfree(d_r_src, st); dfree(d_r_hidx, st); dfree(d_r_widx, st);
        dfree(d_r_aidx, st); dfree(d_lstate, st); dfree(d_work, st); dfree(d_nwork, st); dfree(d_nsusp, st);
        dfree(d_pcost, st); dfree(d_hflag, st); dfree(d_heavy, st); dfree(d_hbins, st);
        dfree(d_susp_a, st); dfree(d_susp_b, st); dfree(d_pool_a, st); dfree(d_pool_b, st); dfree(d_pool_used, st);
        dfree(d_prof, st);
        dfree(d_fill_state, st); dfree(d_fill_work, st); dfree(d_nfill, st);
        dfree(d_ls_key, st); dfree(d_ls_n, st); dfree(d_ls_rep, st); dfree(d_ls_slot, st);
        dfree(d_ls_rep_work, st); dfree(d_ls_dup, st); dfree(d_ls_left, st); dfree(d_ls_ok, st);
        for (auto &b : scan_tmp) dfree(b, st);
        cudaStreamSynchronize(st);
        cudaStreamDestroy(st);
    }
    for (auto &e : ev)
        if (e) cudaEventDestroy(e);
    if (status != PJG_OK) {
        delete res;
        return status;
    }
    *out = res;
    return PJG_OK;
}

extern "C" {

int64_t pjg_results_count(const pjg_results *r) { return r ? r->store.hits : 0; }

int64_t pjg_results_atom_count(const pjg_results *r) { return r ? r->store.atoms : 0; }

pjg_status pjg_results_copy(const pjg_results *r, int32_t *structure, int32_t *template_index, int64_t *ordinal,
                            double *rmsd, double *rotation, double *centres, int64_t *atom_offset, int32_t *atoms) {
    if (!r) return fail(PJG_ERR_INVALID, "null results");
    if (r->count_only) return fail(PJG_ERR_INVALID, "the results of a count-only query hold no hits");
    const HitStore &hs = r->store;
    const size_t n = (size_t)hs.hits;
    if (atom_offset) atom_offset[n] = hs.atoms;
    if (n == 0) return PJG_OK;
    int prev = 0;
    cudaGetDevice(&prev);
    if (prev != r->device) cudaSetDevice(r->device);
    cudaError_t e = copy_out_all({{structure, hs.structure, 4 * n},
                                  {template_index, hs.tpl, 4 * n},
                                  {ordinal, hs.ordinal, 8 * n},
                                  {rmsd, hs.rmsd, 8 * n},
                                  {rotation, hs.rot, 72 * n},
                                  {centres, hs.centres, 48 * n},
                                  {atom_offset, hs.atom_offset, 8 * n},
                                  {atoms, hs.atoms_, 4 * (size_t)hs.atoms}});
    if (prev != r->device) cudaSetDevice(prev);
    if (e != cudaSuccess) return fail(PJG_ERR_CUDA, "results copy: %s", cudaGetErrorString(e));
    return PJG_OK;
}

int64_t pjg_results_warning_count(const pjg_results *r) { return r ? r->store.warns : 0; }

pjg_status pjg_results_superposed(const pjg_results *r, const pjg_structures *s, double *xyz) {
    if (!r || !s) return fail(PJG_ERR_INVALID, "null argument");
    if (r->count_only) return fail(PJG_ERR_INVALID, "the results of a count-only query hold no hits");
    if (s != r->structures) return fail(PJG_ERR_INVALID, "structures differ from the ones the query searched");
    const HitStore &hs = r->store;
    if (hs.atoms == 0) return PJG_OK;
    if (!xyz) return fail(PJG_ERR_INVALID, "null output");
    int prev = 0;
    cudaGetDevice(&prev);
    if (prev != r->device) cudaSetDevice(r->device);
    cudaStream_t st = nullptr;
    double *d_out = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&d_out, (size_t)hs.atoms * 3 * sizeof(double), st);
    if (e == cudaSuccess) {
        launch_superposed_atoms(st, hs.hits, hs.atoms, hs.structure, hs.atom_offset, hs.atoms_, hs.rot, hs.centres,
                                s->d_atom_base, s->d_xyz64, d_out);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(xyz, d_out, (size_t)hs.atoms * 3 * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (d_out) cudaFreeAsync(d_out, st);
    if (st) {
        cudaError_t e2 = cudaStreamSynchronize(st);
        if (e == cudaSuccess) e = e2;
        cudaStreamDestroy(st);
    }
    if (prev != r->device) cudaSetDevice(prev);
    if (e != cudaSuccess) return fail(PJG_ERR_CUDA, "superposed atoms: %s", cudaGetErrorString(e));
    return PJG_OK;
}

pjg_status pjg_results_warnings(const pjg_results *r, int32_t *structure, int64_t *hits_before) {
    if (!r) return fail(PJG_ERR_INVALID, "null results");
    if (r->count_only) return fail(PJG_ERR_INVALID, "the results of a count-only query hold no warnings");
    const HitStore &hs = r->store;
    if (hs.warns == 0) return PJG_OK;
    int prev = 0;
    cudaGetDevice(&prev);
    if (prev != r->device) cudaSetDevice(r->device);
    cudaError_t e = copy_out(structure, hs.warn_structure, 4 * (size_t)hs.warns);
    if (e == cudaSuccess) e = copy_out(hits_before, hs.warn_before, 8 * (size_t)hs.warns);
    if (prev != r->device) cudaSetDevice(prev);
    if (e != cudaSuccess) return fail(PJG_ERR_CUDA, "warnings copy: %s", cudaGetErrorString(e));
    return PJG_OK;
}

pjg_status pjg_results_stats(const pjg_results *r, pjg_stats *stats) {
    if (!r || !stats) return fail(PJG_ERR_INVALID, "null argument");
    *stats = r->stats;
    return PJG_OK;
}

void pjg_results_destroy(pjg_results *r) {
    if (!r) return;
    int prev = 0;
    cudaGetDevice(&prev);
    const bool other = r->store.cap_h + r->store.cap_w > 0 && prev != r->device;
    if (other) cudaSetDevice(r->device);
    delete r;
    if (other) cudaSetDevice(prev);
}

}  // extern "C"
