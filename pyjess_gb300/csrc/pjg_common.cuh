// pjg_common.cuh — data layouts shared by the host orchestration and the
// kernels of libpjg.
//
// Device layout (HBM):
//   structures  : xyz64  double[3N]      FP64 coordinates as given
//                 xyz32  float4[N]       x,y,z relative to the structure's
//                                        centroid (FP32), w = packed key
//                 name   u32[N]          4 name bytes, a-z upper-cased
//                 sorted i32[N]          atoms by (residue name, serial)
//                 buckets                per structure: residue name u32 and
//                                        [begin,end) into `sorted`
//   templates   : per atom: signature id, FP64 position, weight, key bits
//                 per template: n x n distance matrix (FP64)
//                 per query: n x n annulus parameters (FP64 + FP32 bounds)
//   candidate lists, per (structure, signature) of a structure chunk:
//                 cand order : i32 atom (level-0 seeds; points from xyz32)
//                 leaf order : i32 atom + float4 (levels >= 1), the order
//                              in which the reference's kd-tree DFS reports
//                              accepted leaves; only for the lists put in
//                              leaf order, packed in request order
#pragma once

#include <cstdint>

namespace pjg {

// A candidate key packs (residue number, chainID2) for the chain/residue
// rules of TessTemplate_check: key = (resSeq << 8) | chainID2.
__host__ __device__ inline int32_t make_key(int32_t resseq, uint8_t chain2) {
    return (int32_t)((uint32_t)resseq << 8) | (int32_t)chain2;
}

// Candidate-rule kinds of a signature (see the match rules in
// pjg_api.cu: build_signatures).
enum Rule : int32_t {
    RULE_ANY = 0,
    RULE_NAME = 1,
    RULE_NAME_OR_PARTNER = 2,
    RULE_NAME_OR_MAINCHAIN = 3,
    RULE_ELEMENT = 4,
};

// Annulus parameters between an earlier-level template atom p and a later
// one q (Scanner_next, patches/Scanner.c.patch:308-325, and Annulus_reuse,
// patches/Annulus.c.patch:107-139).  FP64 values are the reference's exact
// squared radii; the FP32 bounds bracket them with the guard band:
//   d2 < lo_rej or d2 > hi_rej           -> certainly outside
//   lo_acc <= d2 <= hi_acc               -> certainly inside
//   otherwise                            -> FP64 recheck
struct AnnulusParam {
    float4 thr;        // lo_rej, lo_acc, hi_acc, hi_rej (FP32, squared)
    double a2, b2, b;  // exact squared radii and the outer radius
    double pad;
};

// Per-query device pointers of one structure chunk.
struct ChunkView {
    // structures (chunk-relative indices s in [0, n_structures))
    int32_t n_structures;
    const int64_t *atom_base;     // [S] first atom (global index)
    const int32_t *atom_count;    // [S]
    const double *xyz64;          // global atom indexing
    const float4 *xyz32;
    const uint32_t *name;
    const uint32_t *resname;
    const int32_t *sorted;        // global, values are structure-local
    const int32_t *bucket_begin;  // [S+1] into bucket arrays
    const uint32_t *bucket_name;
    const int32_t *bucket_lo;     // structure-local positions into sorted
    const int32_t *bucket_hi;
    int64_t n_atoms;              // atoms of the whole structure set
    const uint32_t *lrank;        // [3][n_atoms] strict-lower axis rank
    const uint32_t *urank;        // [3][n_atoms] unique axis rank
    // distinct atom names of each residue bucket (global bucket index) with
    // their atom counts: [nh_begin[b], nh_begin[b + 1]) into nh_name/nh_count
    const int32_t *nh_begin;
    const uint32_t *nh_name;
    const int32_t *nh_count;
    const uint8_t *name_id;       // per atom: index of its name among its
                                  // bucket's distinct names (255 past 254)
    // per distinct name of a bucket (same indexing as nh_name): start of its
    // atoms in nh_pos, structure-local; nh_pos holds each structure's atoms
    // grouped by (bucket, name), each group in ResIndex order
    const int32_t *nh_off;
    const int32_t *nh_pos;
};

struct SigView {
    int32_t n_sigs;
    const int32_t *code;
    const int32_t *rule;
    const int32_t *mainchain;       // template lists a main-chain name
    const int32_t *name_begin;      // [G+1]
    const uint32_t *names;
    const int32_t *res_begin;       // [G+1] deduplicated residue names
    const uint32_t *resnames;
    const int32_t *partner_begin;   // [G+1]
    const uint32_t *partner_res;
    const uint32_t *partner_name;
};

struct TemplateView {
    int32_t n_templates;
    int32_t max_atoms;
    const int32_t *atom_begin;      // [T+1]
    const int32_t *sig;             // [A]
    const double *pos;              // [3A]
    const int32_t *key;             // [A] make_key(resSeq, chainID2)
    const int32_t *param_begin;     // [T+1] into params (n*n each)
    const AnnulusParam *params;
};

struct CandView {
    int32_t n_sigs;                 // lists are indexed [s * n_sigs + g]
    const int32_t *count;           // |C|
    const int64_t *offset;          // start in cand_atom
    const int32_t *cand_atom;       // structure-local atom, candidate order
    const int64_t *leaf_offset;     // start in the leaf arrays (ordered lists)
    const int32_t *leaf_atom;       // structure-local atom, kd leaf order
    const float4 *leaf_xyz;         // its FP32 point (xyz32)
    const int64_t *blk_offset;      // first block of the list
    const float4 *blk_lo;           // bounding box of each block of CULL_BLK
    const float4 *blk_hi;           //   consecutive leaves (FP32)
};

// Counters accumulated by the kernels (int64, device).
enum Counter : int {
    C_PAIRS = 0,
    C_SCANNED,
    C_CAND,
    C_PARTIALS,
    C_COMPLETE,
    C_PASSING,
    C_RECHECK,
    C_BYTES_CAND,
    C_BYTES_EXP,
    C_BYTES_SUP,
    C_OVERFLOW,       // complete-row buffer overflow (rows dropped)
    C_PASS_OVERFLOW,  // passing-row buffer overflow
    C_LEAF_EXACT,     // lists ordered by the exact sequential replay
    C_LEAF_SORTED,    // lists ordered by sorted axes
    C_LEAF_REPLAY,    // kd nodes replayed by qselect in the sorted-axis path
    C_LEAF_LISTS,     // lists put in kd leaf order
    C_LEAF_ENTRIES,   // entries of those lists
    C_ERROR,          // error code: 7 an unordered list of a template over
                      // 32 atoms (internal), 2 frontier tile too
                      // small, 3 time budget exhausted, 4 leaf order: too many
                      // small subtrees, 5 a partition did not converge, 6 an
                      // inconsistent node partition (0 = none)
    C_LEAF_SHARED,    // requested lists sharing another list's leaf order
    C_NUM
};

}  // namespace pjg
