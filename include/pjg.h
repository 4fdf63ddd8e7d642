/*
 * pjg.h — C ABI of the GB300 template-matching library (libpjg.so).
 *
 * This is the boundary a host binding calls instead of the Jess C API that
 * PyJess's Cython layer drives.  The reference consumes, per molecule and one
 * candidate at a time:
 *
 *   Jess_create / Jess_addTemplate / Jess_free     include/jess/jess.pxd:18-21
 *   Jess_query(J, M, t, s, reorder)                include/jess/jess.pxd:22
 *   JessQuery_next / JessQuery_nextTemplate        include/jess/jess.pxd:24-25
 *   JessQuery_template / JessQuery_atoms           include/jess/jess.pxd:26-27
 *   JessQuery_superposition                        include/jess/jess.pxd:28
 *   Superposition_rmsd / _rotation / _centroid     include/jess/super.pxd:7-14
 *
 * and replays the candidate automaton of Query.__next__
 * (src/pyjess/_jess.pyx:2197-2283) on top.  This library instead takes whole
 * batches (every template against every structure), runs the search on the
 * GPU and returns the final, ordered hit list of each structure, with the
 * automaton (rmsd filter, NaN-rotation skip, best_match, max_candidates)
 * already applied.  Plain C types only; every call returns a pjg_status and
 * never throws.  Handles are immutable after creation and may be shared by
 * threads; each pjg_query call runs on its own stream with its own scratch.
 */
#ifndef PJG_H
#define PJG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    PJG_OK = 0,
    PJG_ERR_INVALID = 1,       /* malformed input or parameter            */
    PJG_ERR_OOM = 2,           /* device or host allocation failed        */
    PJG_ERR_CUDA = 3,          /* CUDA runtime error (message available)  */
    PJG_ERR_NO_DEVICE = 4,     /* no CUDA device visible                  */
    PJG_ERR_TIMEOUT = 5,       /* a kernel's bounded work loop ran out    */
    PJG_ERR_CAPACITY = 6       /* an internal buffer limit was exceeded   */
} pjg_status;

/* ignore_chain modes, as the reference's IgnoreType
 * (patches/Template.h.patch:17 ignoreNone, ignoreResidues, ignoreAtoms). */
enum { PJG_IGNORE_NONE = 0, PJG_IGNORE_RESIDUES = 1, PJG_IGNORE_ATOMS = 2 };

/* precision / launch modes of pjg_query */
enum {
    /* FP64 distance tests, one structure per launch sequence: the plain
     * GPU method the batched path is measured against. */
    PJG_MODE_PLAIN_FP64 = 0,
    /* all pairs in one launch sequence; distance tests in FP32 on
     * centroid-relative coordinates with a guard band, anything inside the
     * band rechecked in FP64 with the reference's operation order. */
    PJG_MODE_BATCHED_FP32 = 1,
    /* all pairs in one launch sequence, FP64 distance tests. */
    PJG_MODE_BATCHED_FP64 = 2
};

/*
 * Templates, packed.  T templates with A atoms in total; template t owns
 * atoms [atom_offset[t], atom_offset[t+1]).  Each template atom carries the
 * fields of the reference's TessAtom (patches/TessAtom.h.patch:31-44):
 * match code, residue number, chain characters, position, distance weight,
 * atom-name alternatives and residue-name alternatives.  Names are 4 bytes,
 * encoded as in the reference ('_' for blanks, residue names 3 chars + NUL).
 * Corresponds to Template.__init__ / TemplateAtom.__init__
 * (src/pyjess/_jess.pyx:1399-1495, 1825-1912) plus Jess_addTemplate.
 */
typedef struct {
    int32_t n_templates;
    const int32_t *atom_offset;      /* [T+1]                              */
    const int32_t *code;             /* [A] match mode                     */
    const int32_t *res_seq;          /* [A]                                */
    const uint8_t *chain;            /* [A*2] chainID1, chainID2           */
    const double *xyz;               /* [A*3]                              */
    const double *dist_weight;       /* [A]                                */
    const int32_t *name_offset;      /* [A+1] into names                   */
    const uint8_t *names;            /* [*4]                               */
    const int32_t *resname_offset;   /* [A+1] into resnames                */
    const uint8_t *resnames;         /* [*4]                               */
    const int32_t *dim;              /* [T] number of distinct residues    */
} pjg_template_set;

/*
 * Structures (molecules), packed.  S structures with N atoms in total;
 * structure s owns atoms [atom_offset[s], atom_offset[s+1]).  Only the Atom
 * fields the search reads (patches/Atom.h.patch:7-26): coordinates, serial,
 * name, residue name, chain characters, residue number.
 * Corresponds to Molecule.__init__ (src/pyjess/_jess.pyx:632-684).
 */
typedef struct {
    int32_t n_structures;
    const int64_t *atom_offset;      /* [S+1]                              */
    const double *xyz;               /* [N*3]                              */
    const uint8_t *name;             /* [N*4]                              */
    const uint8_t *resname;          /* [N*4] 3 chars + NUL                */
    const uint8_t *chain;            /* [N*2]                              */
    const int32_t *res_seq;          /* [N]                                */
    const int32_t *serial;           /* [N]                                */
} pjg_structure_set;

/* Query parameters: the arguments of Jess.query
 * (src/pyjess/_jess.pyx:2758-2869) plus the GPU execution mode. */
typedef struct {
    double rmsd_threshold;
    double distance_cutoff;          /* Jess_query t                       */
    double max_dynamic_distance;     /* Jess_query s                       */
    int32_t max_candidates;          /* -1: unlimited                      */
    int32_t ignore_chain;            /* PJG_IGNORE_*                       */
    int32_t best_match;              /* 0/1                                */
    int32_t reorder;                 /* 0/1                                */
    int32_t mode;                    /* PJG_MODE_*                         */
    double guard_band;               /* Angstrom, FP32 mode (0: 1e-4)      */
    int32_t count_only;              /* 1: count the hits and warnings
                                        (pjg_results_count, _atom_count,
                                        _warning_count, stats) without
                                        keeping them; copying them out
                                        then returns PJG_ERR_INVALID.  For
                                        queries whose hits outgrow memory */
} pjg_query_params;

/* Per-query counters and device timings (milliseconds, CUDA events). */
typedef struct {
    int64_t pairs;                   /* template x structure pairs         */
    int64_t candidate_entries;       /* sum of candidate-list lengths      */
    int64_t partials;                /* partial assignments generated      */
    int64_t complete;                /* complete assignments (all atoms)   */
    int64_t passing;                 /* complete with rmsd <= threshold    */
    int64_t hits;                    /* after the automaton                */
    int64_t fp64_rechecks;           /* guard-band rechecks (FP32 mode)    */
    int64_t leaf_exact;              /* lists ordered by the exact replay  */
    int64_t leaf_sorted;             /* lists ordered by sorted axes       */
    int64_t leaf_replays;            /* kd nodes replayed there (ties)     */
    int64_t bytes_candidates;        /* algorithmic bytes, candidate stage */
    int64_t bytes_expansion;         /* algorithmic bytes, expansion stage */
    int64_t bytes_superposition;     /* algorithmic bytes, superposition   */
    double ms_candidates;
    double ms_expansion;
    double ms_superposition;
    double ms_total;                 /* device time of the whole query     */
    int32_t launches;                /* kernels launched by the query      */
    int32_t chunks;                  /* structure chunks processed         */
    int64_t leaf_lists;              /* lists put in kd leaf order         */
    int64_t leaf_entries;            /* entries of those lists             */
    int64_t suspensions;             /* pair searches stopped at a list
                                        with no leaf order yet (rerun)     */
    int32_t search_rounds;           /* search launches                    */
    int32_t row_splits;              /* chunks redone on fewer structures
                                        because their complete rows did
                                        not fit in memory                  */
    int64_t leaf_shared;             /* of leaf_lists: lists of the same
                                        atoms as another list of their
                                        structure, sharing its leaf order  */
} pjg_stats;

typedef struct pjg_templates pjg_templates;
typedef struct pjg_structures pjg_structures;
typedef struct pjg_results pjg_results;

/* Library / device --------------------------------------------------------*/

/* Replaces nothing (the reference has no device); returns PJG_OK and the
 * device ordinal in use, or PJG_ERR_NO_DEVICE. */
pjg_status pjg_init(int32_t device);

/* Last error message of the calling thread (never NULL). */
const char *pjg_last_error(void);

/* Templates ---------------------------------------------------------------*/

/* Replaces Jess_create + Jess_addTemplate per template + TessTemplate_copy
 * (patches/Jess.c.patch:63-72, patches/TessTemplate.c.patch:265-337).
 * Builds the distance matrices (TessAtom_distance, patches/TessAtom.c.patch
 * :229-244), the per-pair annulus radii and the candidate signatures, and
 * uploads them.  Template t keeps index t; the search visits templates in
 * reverse index order as the reference's prepend-list does. */
pjg_status pjg_templates_create(const pjg_template_set *set, pjg_templates **out);

/* Replaces Jess_free (patches/Jess.c.patch:52-61). */
void pjg_templates_destroy(pjg_templates *t);

/* Structures --------------------------------------------------------------*/

/* Replaces Molecule creation + ResIndex_create (patches/ResIndex.c.patch
 * :24-119, src/pyjess/_jess.pyx:632-684): sorts each structure's atoms by
 * (residue name, serial), builds the residue buckets and the FP64 and
 * centroid-relative FP32 coordinate arrays, uploads them and ranks every
 * atom along each axis on the device (the kd leaf order's sorted-axis path).
 * A non-finite coordinate returns PJG_ERR_INVALID (the reference accepts
 * one: there a NaN atom passes every distance test). */
pjg_status pjg_structures_create(const pjg_structure_set *set, pjg_structures **out);

/* Replaces Molecule_free. */
void pjg_structures_destroy(pjg_structures *s);

/* Query -------------------------------------------------------------------*/

/* Replaces Jess_query + the JessQuery_next / Scanner_next loop +
 * JessQuery_superposition + the Query.__next__ automaton
 * (patches/Jess.c.patch:74-216, patches/Scanner.c.patch:110-336,
 * src/pyjess/_jess.pyx:2197-2283) for every structure of `s` against every
 * template of `t`, all on the device.  Results are ordered by structure,
 * then by template in reverse index order, then by the reference's
 * candidate order. */
pjg_status pjg_query(const pjg_templates *t, const pjg_structures *s,
                     const pjg_query_params *params, pjg_results **out);

/* Number of hits in total and the number of template atoms of hit i's
 * template (the length of its atom list). */
int64_t pjg_results_count(const pjg_results *r);
/* Sum over hits of the template atom count (size of the atom index array). */
int64_t pjg_results_atom_count(const pjg_results *r);

/* Copy the hits out (host arrays; the hits stay on the device until
 * pjg_results_destroy).  Each array may be NULL to skip it.
 *   structure[i], template_index[i]    which pair hit i belongs to
 *   ordinal[i]     position of hit i in its pair's candidate stream
 *   rmsd[i]        Superposition_rmsd
 *   rotation[9i]   Superposition_rotation (row major, molecule -> template)
 *   centres[6i]    Superposition_centroid(0) then (1): molecule, template
 *   atom_offset[i] start of hit i in atoms (size count+1)
 *   atoms[]        structure-relative atom indices, in template atom order
 *                  (JessQuery_atoms, patches/Jess.c.patch:121-126) */
pjg_status pjg_results_copy(const pjg_results *r, int32_t *structure,
                            int32_t *template_index, int64_t *ordinal,
                            double *rmsd, double *rotation, double *centres,
                            int64_t *atom_offset, int32_t *atoms);

/* NaN-rotation events that Query.__next__ reports as UserWarning
 * (src/pyjess/_jess.pyx:2238-2251): for each event, the structure and the
 * number of hits of that structure that precede it. */
int64_t pjg_results_warning_count(const pjg_results *r);
pjg_status pjg_results_warnings(const pjg_results *r, int32_t *structure,
                                int64_t *hits_before);

/* Replaces, for every hit at once, Hit.atoms(transform=True) /
 * Molecule.transform(hit.transformation) of the reference
 * (src/pyjess/_jess.pyx:878-907, 2343-2377): each hit's matched molecule
 * atoms mapped into its template's frame, T(v) R T(-c) x, computed on the
 * device from the structures `s` the query searched (any other set returns
 * PJG_ERR_INVALID).  xyz[3k + d] for hit atom k, in the order of
 * pjg_results_copy's atoms (pjg_results_atom_count x 3 doubles). */
pjg_status pjg_results_superposed(const pjg_results *r, const pjg_structures *s, double *xyz);

/* Counters and device timings of the query that produced `r`. */
pjg_status pjg_results_stats(const pjg_results *r, pjg_stats *stats);

void pjg_results_destroy(pjg_results *r);

/* Execution tuning -------------------------------------------------------
 *
 * No counterpart in the reference (its search is one thread).  The knobs of
 * the GPU search that trade work between kernels; the autotuner
 * (pyjess_gb300/tune.py) measures them on a sample of a workload and sets
 * the fastest.  Process-wide: each pjg_query reads the values in force when
 * it starts.  A field of 0 keeps the built-in default.
 *   leaf_levels    levels (after level 0) whose candidate lists are put in
 *                  kd leaf order before the search; deeper lists when a
 *                  pair first reaches them (default 4; -1 every list up
 *                  front; the plain FP64 mode always orders every list)
 *   block_min      shortest list the search expands one parent at a time
 *                  with block culling (shorter lists: lanes over (parent,
 *                  candidate) pairs) (default 64, 1 .. 65535)
 *   tile_cap       most entries of a frontier tile (default 4096, 32 ..
 *                  16384)
 *   pair_grain     (structure, template) pairs a search warp takes from the
 *                  work queue at a time (default 1, 1 .. 64)
 *   leaf_rank_max  longest tie-free list put in leaf order by the
 *                  leaf-order kernel's instance with the smallest buffers
 *                  (longer lists: the instances for up to 512 and 1024
 *                  entries) (default 256, 1 .. 256)
 *   leaf_reach     when a pair reaches a list with no leaf order it is
 *                  suspended and requests that list and the next
 *                  leaf_reach - 1 deeper ones of its levels (-1, the
 *                  default: every deeper one; 1 .. 64)
 * Out-of-range values return PJG_ERR_INVALID and change nothing. */
typedef struct {
    int32_t leaf_levels;
    int32_t block_min;
    int32_t tile_cap;
    int32_t pair_grain;
    int32_t leaf_rank_max;
    int32_t leaf_reach;
} pjg_tuning;

/* Set the tuning (NULL restores every default). */
pjg_status pjg_set_tuning(const pjg_tuning *tuning);
/* The tuning in force, defaults filled in. */
pjg_status pjg_get_tuning(pjg_tuning *tuning);
/* Name of the current CUDA device (the autotuner's cache key). */
pjg_status pjg_device_name(char *buf, int32_t len);

/* Structure ingestion ---------------------------------------------------
 *
 * Replaces the per-record loop of the reference's PDB reader
 * (src/pyjess/_io.py:52-103, PDBMoleculeParser, over the C Atom_parse):
 * scans a whole PDB text and writes every ATOM (and HETATM, unless
 * PJG_PDB_SKIP_HETATM) record up to the first ENDMDL (unless
 * PJG_PDB_IGNORE_ENDMDL) into `records`, 59-byte packed rows of the atom
 * table (x, y, z f64; occupancy, temperature factor f32; serial i32; name
 * 4 B; altloc; residue name 4 B; chain 2 B; residue number i32; insertion
 * code; segment 4 B; element 2 B; charge i8).  Host code; thread-safe.
 * Returns PJG_OK with n_atoms rows and end_offset = where the scan ended
 * (the ENDMDL line, or len).  A record in a form it does not take (blank
 * or non-decimal fields, non-printable bytes, a short line, an mmCIF tag,
 * more records than `capacity`) returns PJG_ERR_INVALID with stop_offset =
 * that line's offset, and the caller reads the text with its general
 * parser. */
enum { PJG_PDB_IGNORE_ENDMDL = 1, PJG_PDB_SKIP_HETATM = 2 };
pjg_status pjg_parse_pdb(const char *text, int64_t len, int32_t flags, void *records, int64_t capacity,
                         int64_t *n_atoms, int64_t *end_offset, int64_t *stop_offset);

/* Allocation-free superposition --------------------------------------------
 *
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory while they run (real-time loops that must not block on the
 * allocator, applications whose memory manager owns every device
 * allocation).  It superposes n_rows candidate assignments
 * of one template: row r's molecule atoms are mol_xyz[(r*n_atoms + k)*3 + d],
 * the template's atoms tpl_xyz[3k + d] (k = template atom, 1 <= n_atoms <=
 * 32), all device pointers.  It writes, per row, rmsd[r], rotation[9r..]
 * (row major, molecule -> template) and centres[6r..] (molecule centroid,
 * template centroid), then pass_rows[0 .. *pass_count) = the rows with
 * rmsd <= rmsd_threshold (and a defined rotation, n_atoms >= 3) in row order.
 * Kernels are enqueued on `stream` (a cudaStream_t, NULL for the default
 * stream); the call returns without waiting.
 *
 * It allocates nothing: its scratch is a static device array of
 * PJG_NOALLOC_MAX_ROWS (2^20) row flags (4 MiB) that every GPU loading the
 * library keeps until the process exits.  More rows than that, or a bad
 * argument, return PJG_ERR_INVALID with a message from
 * pjg_noalloc_last_error().  The first call on each device looks up that
 * array's device address with the device current; make that first call
 * before any stream capture.  The address is kept per device together with
 * the id of the CUDA context it belongs to: after the context is reset
 * (cudaDeviceReset), the next call looks it up again, so that call too
 * should come before any stream capture.  All calls share the array: calls
 * that overlap on the GPU race, so serialise them. */
#define PJG_NOALLOC_MAX_ROWS (1 << 20)
pjg_status pjg_superpose_noalloc(const double *mol_xyz, const double *tpl_xyz, int32_t n_rows, int32_t n_atoms,
                                 double rmsd_threshold, double *rmsd, double *rotation, double *centres,
                                 int32_t *pass_rows, int32_t *pass_count, void *stream);
const char *pjg_noalloc_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* PJG_H */
