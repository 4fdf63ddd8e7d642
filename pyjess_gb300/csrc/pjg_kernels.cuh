// pjg_kernels.cuh — kernel declarations and launch argument blocks.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "pjg_common.cuh"

namespace pjg {

// rows one call of pjg_superpose_noalloc may take (its static scratch)
#ifndef PJG_NOALLOC_MAX_ROWS
#define PJG_NOALLOC_MAX_ROWS (1 << 20)
#endif

#ifndef PJG_SEARCH_WARPS
#define PJG_SEARCH_WARPS 8
#endif
constexpr int SEARCH_WARPS = PJG_SEARCH_WARPS;  // warps per block of k_search
// resident k_search blocks per SM the register allocation is sized for
#ifndef PJG_SEARCH_MIN_BLOCKS
#define PJG_SEARCH_MIN_BLOCKS 2
#endif
// leaves per culling block: k_search tests a parent's join box against the
// bounding box of each block of CULL_BLK consecutive leaves of a list in kd
// leaf order, and loads the leaves of the blocks it meets (8, 16 or 32)
#ifndef PJG_CULL_BLK
#define PJG_CULL_BLK 32
#endif
constexpr int CULL_BLK = PJG_CULL_BLK;
static_assert(CULL_BLK == 8 || CULL_BLK == 16 || CULL_BLK == 32, "culling block of 8, 16 or 32 leaves");
// templates of more than 32 atoms: k_search_large, warps per block and
// per-warp shared-memory bytes for templates of up to nmax atoms
constexpr int LARGE_WARPS = 2;
__host__ __device__ constexpr int large_warp_bytes(int nmax) { return ((52 * nmax) + 15) & ~15; }
// longest template pjg_templates_create accepts
constexpr int MAX_TEMPLATE_ATOMS = 1024;
// kd leaf order of tie-free lists: axis partitions (k_leaf_part), or with
// -DPJG_LEAF_RANK=1 the rank method (k_leaf_order)
#ifndef PJG_LEAF_RANK
#define PJG_LEAF_RANK 0
#endif
constexpr int LEAF_WARPS = 4;          // warps per block of k_leaf_order
#if PJG_LEAF_RANK
constexpr int LEAF_FAST_MAX = 192;     // capacity of the rank method's buffers
constexpr int LEAF_RANK_MAX = 192;     // default: longest list ordered by the rank method
#else
constexpr int LEAF_FAST_MAX = 256;     // capacity of k_leaf_part's first instance
constexpr int LEAF_RANK_MAX = 256;     // default: longest list that instance takes
#endif
// longest tie-free list ordered by axis partitions (256, 512 or 1024; the
// longer ones by sorted axes)
#ifndef PJG_PART_MAX
#define PJG_PART_MAX 1024
#endif
constexpr int PART_MAX = PJG_PART_MAX;
static_assert(PART_MAX == 256 || PART_MAX == 512 || PART_MAX == 1024, "axis partitions up to 256, 512 or 1024");
// kernels one launch_leaf_order call launches
constexpr int LEAF_ORDER_LAUNCHES = PJG_LEAF_RANK ? 7 : (PART_MAX >= 1024 ? 8 : PART_MAX >= 512 ? 7 : 6);
constexpr int LEAF_LISTS = 5;          // leaf-order worklists: three k_leaf_sorted size
                                       //   classes and two forwarded size classes
constexpr int LEAF_MID_MAX = 384;      // longest list of the rank method's larger instance
constexpr int LEAF_SORT_FROM = 64;     // rank method: a level's nodes of this many entries or
                                       //   more are ordered by a bitmap sort
constexpr int LEAF_SORT_WORDS = 128;   // its window (32-bit words)
constexpr int LEAF_SORTED_MAX = 2048;  // longest list ordered by sorted axes
constexpr int LEAF_SORT_MAX = 1024;    // longest list ordered by presorted axes
constexpr int EXACT_MAX = 4096;        // longest list replayed warp-parallel

// Search profile: event counts and clock64 cycles of k_search's sections,
// summed over warps.  Compiled only with -DPJG_SEARCH_PROF=1 (a separate
// library variant used to explain the kernel's cost; the timed build has
// none of it).
#ifndef PJG_SEARCH_PROF
#define PJG_SEARCH_PROF 0
#endif
enum SearchProf : int {
    SP_PAIRS = 0,        // pairs taken from the queue
    SP_EMPTY,            // pairs with an empty candidate list
    SP_CYC_PAIR,         // cycles from taking a pair to finishing it
    SP_CYC_SETUP,        // cycles of a pair's set-up (lengths, order, levels)
    SP_CYC_SEED,         // cycles filling level-0 tiles
    SP_CYC_BLOCK,        // cycles in block-mode expansions
    SP_CYC_PROD,         // cycles in product-mode expansions
    SP_CYC_EMIT,         // cycles in emit (inside the two above)
    SP_LOOP_ITERS,       // iterations of the depth-first loop
    SP_BLOCK_VISITS,     // block-mode visits of a parent
    SP_BLOCK_VISITS_L0,  //   of which from level 0
    SP_CHAIN_FULL,       // parent chains gathered by walking the tiles
    SP_CHAIN_SIBLING,    // parent chains reused from a sibling
    SP_G0_ITERS,         // 32-block steps of the block scan
    SP_BLOCKS_TESTED,    // block boxes tested against the join box
    SP_BLOCKS_HIT,       // blocks whose box meets the join box
    SP_LEAVES_INBOX,     // leaves inside the join box (queued)
    SP_BATCHES,          // full-test batches
    SP_BATCH_LANES,      // queued leaves fully tested
    SP_CHILD_BLOCK,      // children / rows from block mode
    SP_PROD_BATCHES,     // product-mode batches
    SP_PROD_BATCHES_L0,  //   of which from level 0
    SP_PROD_LANES,       // (parent, candidate) tests in product mode
    SP_CHILD_PROD,       // children / rows from product mode
    SP_FP64,             // candidates decided in FP64
    SP_ROWS,             // complete rows emitted
    SP_CYC_CHAIN,        // cycles gathering a block-mode parent's chain and box
    SP_CYC_BATCH,        // cycles in block-mode full-test batches
    SP_CYC_CTRL,         // cycles of the loop's level bookkeeping (moving up
                         // or down a level, choosing the expansion mode)
    SP_CYC_SUSP,         // cycles suspending pairs (state saved, lists requested)
    SP_TAIL_NS,          // per launch, summed: ns from the first warp finding the
                         // work queue empty to the last warp's exit
    SP_PAIR_MAX_CYC,     // most cycles one pair took (a maximum, not a sum)
    SP_NUM
};

// Leaf-order profile (same build flag): k_leaf_order's section cycles and
// the lists it takes by length class, summed over warps of both instances.
enum LeafProf : int {
    LP_LISTS = 0,        // lists ordered by the rank method
    LP_ENTRIES,          //   their entries
    LP_HANDED,           // lists handed on (longer, or a median tie)
    LP_CYC_LIST,         // cycles of every list begun, load to write-out or hand-on
    LP_CYC_LOAD,         //   loading ranks
    LP_CYC_SORT,         //   bitmap-sorted levels
    LP_CYC_COUNT,        //   counted levels
    LP_CYC_SEG,          //   tie checks, next keys, child nodes
    LP_CYC_WRITE,        //   leaves and block boxes written
    LP_SORT_NODES,       // nodes bitmap-sorted
    LP_SORT_WORDS,       //   bitmap words they cleared and scanned
    LP_COUNT_PAIRS,      // key comparisons of the counted levels
    LP_CLASS,            // lists by length: <=16, <=32, <=64, <=96, <=128,
                         //   <=192, <=384 (7 counters)
    LP_CLASS_ENT = LP_CLASS + 7,  // entries by the same classes (7)
    LP_CLASS_CYC = LP_CLASS_ENT + 7,  // cycles by the same classes (7)
    LP_NUM = LP_CLASS_CYC + 7
};

struct SearchArgs {
    int32_t n_pairs;                   // chunk structures x templates
    int32_t ignore_chain;
    int32_t reorder;
    int32_t best_match;
    int32_t max_candidates;
    int32_t warp_smem;                 // bytes of shared memory per warp
    int32_t cut_inline;                // apply the max_candidates cut while
                                       // searching (non-best mode)
    double rmsd_threshold;
    uint64_t budget_ns;                // per-warp wall-time budget (globaltimer)
    unsigned long long *prof;          // [SP_NUM] search profile (profile
                                       // builds only, else nullptr)
    int32_t block_min;                 // shortest child list expanded one
                                       // parent at a time in block mode
                                       // (shorter: product mode)
    int32_t tile_cap;                  // most entries of a frontier tile
    int32_t pair_grain;                // work-queue items a warp takes at once
    int32_t leaf_reach;                // lists a suspending pair requests: its
                                       // level and the next leaf_reach - 1
                                       // (< 0: every deeper level)
};

// A pair whose search stopped at a level whose candidate list had no kd
// leaf order yet.  Once the list is ordered the pair resumes from its saved
// search state (`state` >= 0: byte offset into the state pool of the round
// that suspended it) or, when the pool was full, runs again from its
// beginning, skipping the `skip` complete rows it has already emitted (the
// search is deterministic, so the replay emits the same rows in the same
// order).
struct Suspended {
    int32_t pair;
    int32_t pad;
    int64_t skip;
    int64_t state;
};

// Saved search state of a suspended pair (16-byte aligned in the pool):
// this header, then per level 0..lev an int4 (F, cnt, par, cnd), then the
// used entries of those levels' tiles.
struct SavedPair {
    int32_t root;
    int32_t lev;
    int64_t emitted;
    int64_t cut_base;
    unsigned long long rechecks;
};

// Lists put in kd leaf order on demand.  state[w] per list of the chunk:
// 0 no leaf order, 1 requested (in `work`), 2 ordered.  state == nullptr:
// every list is ordered.
struct LeafDemand {
    int32_t *state;
    int64_t *work;                     // requested lists, appended
    unsigned long long *n_work;
    const Suspended *resume;           // pairs of this search round;
    int32_t n_resume;                  //   nullptr: pairs 0 .. n_pairs-1
    Suspended *suspended;              // pairs that stopped at an unordered
    unsigned long long *n_suspended;   //   list in this round
    int64_t *leaf_offset;              // [lists] set at the list's request
    unsigned long long *leaf_used;     // leaf entries reserved (may pass the
                                       //   arrays' capacity: the host grows
                                       //   them before the lists are ordered)
    unsigned char *pool_out;           // states saved in this round
    unsigned long long *pool_used;     //   (bytes taken; may pass pool_cap)
    int64_t pool_cap;
    const unsigned char *pool_in;      // states of the pairs of this round
    // lists filled on demand (nullptr: every list of the chunk is filled
    // before the search): per list 0 not yet, 1 filled or queued
    int32_t *fill_state;
    int64_t *fill_work;                // level-0 lists queued for the fill
    unsigned long long *n_fill;
    // the costliest pairs first (the round that runs every pair): the
    // level demand writes each pair's estimated cost as a power-of-two
    // bucket (0: nothing to search), the pairs above a threshold are listed
    // in `heavy` and taken before the others, which keep their order
    uint8_t *pair_cost;                // [n_pairs] (nullptr: not estimated)
    const int32_t *heavy;              // pairs taken first (nullptr: none)
    const unsigned long long *n_heavy; //   how many
    const uint8_t *heavy_flag;         // [n_pairs] 1: the pair is in `heavy`
};

// Requested lists whose candidate atoms are the same share one kd leaf
// order: a table of list keys (structure, length, hash of the atom set) for
// the chunk, and the worklists of one ordering round.
struct ListShare {
    unsigned long long *key;       // [mask + 1] table keys (0: empty slot)
    int32_t *rep;                  // [mask + 1] the list ordered for the key
                                   //   (-1: none yet; the first to claim it)
    int64_t mask;                  // table size - 1 (a power of two)
    int32_t *slot;                 // [requested lists] table slot of each (-1:
                                   //   table full, ordered on its own)
    int64_t *rep_work;             // lists ordered in this round
    int64_t *dup_work;             // lists sharing another's order: list << 32 | rep
    int64_t *left_work;            // shared lists whose atoms turned out to
                                   //   differ: ordered on their own
    unsigned long long *n;         // [3] lengths of the three worklists
    uint8_t *part_ok;              // [lists] ordered by k_leaf_part (no median
                                   //   tie: the order depends on the set only)
};

// Complete assignments written by k_search.
struct CompleteRows {
    unsigned long long *count;
    int64_t capacity;
    int32_t stride;                    // >= max template atoms
    int32_t *pair;                     // chunk-local pair = s * T + t
    int64_t *ordinal;                  // position in the pair's stream
    int32_t *atoms;                    // [capacity * stride], template order
    double *rmsd;                      // rmsd computed in the search (inline
                                       // cut mode), else nullptr
    int32_t *pair_rows;                // [pairs] complete rows of each pair
};

// Superposition of every complete row, in reference order: row i of pair
// (s, t) with stream ordinal k lands at off_q[s * T + (T - 1 - t)] + k
// (structures ascending, templates descending, then the stream).
struct RowResults {
    const int64_t *off_q;
    int32_t n_templates;
    double *rmsd;
    int32_t *nan_rot;                  // rotation undefined (NaN entries)
    double *rot;                       // [9 * rows]
    double *centres;                   // [6 * rows]
    int64_t *src;                      // complete-row index of each slot
};

// Final hits and warnings of one chunk (Query.__next__ applied on the device).
struct HitSegment {
    int32_t *structure;
    int32_t *tpl;
    int64_t *ordinal;
    double *rmsd;
    double *rot;                       // [9 * hits]
    double *centres;                   // [6 * hits]
    int64_t *atom_offset;              // [hits] first atom of each hit (global)
    int32_t *atoms;
    int32_t *warn_structure;
    int64_t *warn_before;              // hits of the structure before the warning
};

// bytes of k_search's per-warp pair state (shared memory, before the tiles)
size_t search_state_bytes();

// Host-side launchers (the kernels themselves live in pjg_kernels.cu).

void launch_params(cudaStream_t st, int n_templates, const int32_t *atom_begin, const int32_t *param_begin,
                   const double *dist, const double *weight, double r, double s, double g, AnnulusParam *out);

// fill == false: list lengths of every list of the chunk; fill == true: the
// lists themselves, of every list (work == nullptr) or of the lists in
// `work` (claim: only those whose fill state this launch moves from 0 to 1)
void launch_candidates(cudaStream_t st, int blocks, bool fill, const ChunkView &cv, const SigView &sv,
                       int32_t *count, int32_t *scanned, const int64_t *offset, int32_t *cand_atom,
                       const int64_t *work = nullptr, const unsigned long long *n_work = nullptr,
                       int32_t *fill_state = nullptr, bool claim = false);

// exclusive scan of one tile (SCAN_TILE entries) per block
constexpr int SCAN_TILE_THREADS = 512;
constexpr int SCAN_TILE_ITEMS = 2048;
void launch_scan_tiles_i32(cudaStream_t st, const int32_t *in, int64_t n, int64_t *out, int64_t *tile_sums);
void launch_scan_tiles_i64(cudaStream_t st, const int64_t *in, int64_t n, int64_t *out, int64_t *tile_sums);
void launch_scan_add(cudaStream_t st, int64_t *out, int64_t n, const int64_t *tile_offsets);

// kd leaf order of the lists in `work` (n_work entries, read on the device),
// or of every list of the chunk when work == nullptr
#if PJG_SEARCH_PROF
// leaf-order profile: zero it / copy its LP_NUM sums to the host
void leaf_profile_reset(cudaStream_t st);
void leaf_profile_read(unsigned long long *h, cudaStream_t st);
#endif
void launch_leaf_order(cudaStream_t st, int blocks, const ChunkView &cv, int32_t n_sigs, const int32_t *count,
                       const int64_t *offset, const int64_t *blk_offset, const int32_t *cand_atom,
                       const int64_t *leaf_offset, int32_t *leaf_atom, float4 *leaf_xyz, float4 *blk_lo, float4 *blk_hi,
                       int64_t *sorted_list, unsigned long long *sorted_count, int64_t list_cap,
                       int64_t *exact_list, unsigned long long *exact_count, unsigned long long *counters,
                       const int64_t *work, const unsigned long long *n_work, int rank_max,
                       uint8_t *part_ok = nullptr, int count_lists = 1);

// list sharing, around the leaf-order launches of a round: keys of the
// requested lists into the table (and the lists / entries counters), the
// split into lists to order and lists sharing another's order, and after
// the ordering the shared lists pointed at their representatives' leaves and
// blocks once their atoms are checked equal (else queued in left_work)
void launch_list_keys(cudaStream_t st, int blocks, int32_t n_sigs, const int32_t *count, const int64_t *offset,
                      const int32_t *cand_atom, const int64_t *work, const unsigned long long *n_work,
                      const ListShare &ls, unsigned long long *counters);
void launch_list_reps(cudaStream_t st, int blocks, const int64_t *work, const unsigned long long *n_work,
                      const ListShare &ls);
void launch_list_share(cudaStream_t st, int blocks, const ChunkView &cv, int32_t n_sigs, const int32_t *count,
                       const int64_t *offset, const int32_t *cand_atom, int64_t *leaf_offset, int64_t *blk_offset,
                       const ListShare &ls, unsigned long long *counters);

// requests (LeafDemand) the lists of levels 1 .. max_level of every pair
// of the chunk that has no empty candidate list
void launch_demand_levels(cudaStream_t st, int blocks, const TemplateView &tv, const CandView &cd, int32_t n_pairs,
                          int32_t max_level, int32_t reorder, const LeafDemand &dm);
// the pairs whose cost bucket is above the level that leaves at most
// `target` pairs above it: flags and list (n_heavy), from the buckets the
// level demand wrote (bins: 66 counters, zeroed by the caller)
void launch_heavy_pairs(cudaStream_t st, int32_t n_pairs, const uint8_t *pair_cost, unsigned long long *bins,
                        int64_t target, uint8_t *heavy_flag, int32_t *heavy);

// state[work[i]] = 2 for the n_work requested lists
void launch_mark_ordered(cudaStream_t st, int blocks, const LeafDemand &dm);

// per-structure axis ranks (lrank, urank: [3][n_atoms], structure-local
// values); tile_key / tile_idx: scratch of 3 * n_atoms entries
void launch_axis_ranks(cudaStream_t st, int32_t n_structures, const int64_t *atom_base, const int32_t *atom_count,
                       const double *xyz64, int64_t n_atoms, unsigned long long *tile_key, uint16_t *tile_idx,
                       uint32_t *lrank, uint32_t *urank);

// culling blocks per list: ceil(count / CULL_BLK)
void launch_block_counts(cudaStream_t st, int64_t n, const int32_t *count, int32_t *nblk);

// k_search variant: wide = 32-bit frontier entries (structures above 65535
// atoms), fp32 = guarded FP32 distance tests (else exact FP64 throughout)
cudaError_t launch_search(cudaStream_t st, int grid, bool wide, bool fp32, const ChunkView &cv,
                          const TemplateView &tv, const CandView &cd, const SearchArgs &sa, int32_t *pair_counter,
                          const int32_t *scanned, const CompleteRows &out, unsigned long long *counters,
                          const LeafDemand &dm);

// k_search_large over the pairs (chunk structure x templates `large`) of
// the templates with more than 32 atoms; item_counter zeroed by the caller;
// lstate: per-list leaf-order state (nullptr: every list ordered)
cudaError_t launch_search_large(cudaStream_t st, const ChunkView &cv, const TemplateView &tv, const CandView &cd,
                                const SearchArgs &sa, const int32_t *large, int32_t n_large, int32_t *item_counter,
                                const int32_t *scanned, const CompleteRows &out, unsigned long long *counters,
                                const int32_t *lstate);

// every hit atom in its template's frame (out[3 * k + d] for hit atom k)
void launch_superposed_atoms(cudaStream_t st, int64_t n_hits, int64_t n_atoms, const int32_t *structure,
                             const int64_t *atom_offset, const int32_t *atoms, const double *rot,
                             const double *centres, const int64_t *atom_base, const double *xyz64, double *out);

void launch_superpose(cudaStream_t st, int blocks, const ChunkView &cv, const TemplateView &tv,
                      const CompleteRows &in, const RowResults &out);

// reference-order list lengths: cnt_q[s * T + (T - 1 - t)] = pair_rows[s * T + t]
void launch_order_counts(cudaStream_t st, int64_t n_pairs, int32_t n_templates, const int32_t *pair_rows,
                         int32_t *cnt_q);

// Query.__next__ per pair over its rows in reference order: hit / warning
// flags and hit atom counts per row; totals[0..3] += hits, warnings, hit
// atoms, passing rows
void launch_automaton(cudaStream_t st, int64_t n_pairs, int32_t n_templates, const int32_t *atom_begin,
                      const int32_t *cnt_q, const int64_t *off_q, const RowResults &rr, int32_t max_candidates,
                      int32_t best_match, double rmsd_threshold, int32_t *hit, int32_t *warn, int32_t *hit_atoms,
                      unsigned long long *totals);

// compaction of the flagged rows into a HitSegment (hit_idx, warn_idx,
// atom_idx: exclusive scans of the flags / hit atom counts)
void launch_gather_hits(cudaStream_t st, int64_t n_rows, int32_t n_templates, int32_t structure_base,
                        int64_t atom_base, const int32_t *atom_begin, const CompleteRows &in, const RowResults &rr,
                        const int32_t *hit, const int32_t *warn, const int64_t *hit_idx, const int64_t *warn_idx,
                        const int64_t *atom_idx, int32_t best_match, const HitSegment &out);

}  // namespace pjg
