// Kernel declarations and argument blocks of the GB300 motif-extraction engine.
#pragma once

#include "common.cuh"

namespace mtx
{

constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

struct PackArgs
{
    const uint8_t *  raw;          // concatenated sequences
    uint64_t         total;
    const uint32_t * offs;         // nseq + 1 sequence offsets
    uint32_t         nseq;
    const uint8_t *  cmap;         // byte -> symbol code
    int              B;            // bit planes
    uint32_t         l;            // factor length (box 0)
    uint32_t         tml;          // minimum sequence length (shorter ones are skipped)
    uint32_t         vstart;       // first position (relative) at which a match may end
    uint32_t         npat;         // leading pattern sequences (factors only); 0: every sequence is both
    const uint32_t * wstart;       // first factor index of each sequence
    uint8_t *        codes;
    uint32_t *       planes;
    uint32_t         plane_stride;
    uint32_t *       vmask;
    uint32_t *       emask;
    uint32_t *       wpos;
    uint32_t         nblk;
    uint32_t *       err;          // bit 0: a staging wait gave up; bit 1: its drain gave up too
    uint32_t         wait_polls;   // try_wait polls before a staging wait gives up
    uint32_t *       key0;         // null, or the first sort key of every factor (beside wpos): its
    uint32_t         kwin;         // last kwin symbols packed, B bits each, last symbol lowest
};

constexpr uint32_t kStageWaitPolls = 1u << 22;   // default PackArgs::wait_polls

constexpr int kPackThreads = 256;              // 8 warps, each packs 32 blocks of 32 positions
constexpr int kPackCtasPerSm = 4;              // resident CTAs per SM (k_pack's launch bounds)
constexpr uint32_t kPackTile = 8192;           // positions (raw bytes) per staged tile
constexpr int kPackKeyWords = 32 * 33;         // k_pack's per-warp key buffer (dynamic shared memory)

struct FinalizeArgs
{
    uint32_t          U;
    const uint32_t *  u_acc;
    const uint32_t *  v_acc;
    const uint8_t *   split_flags;
    uint32_t          n_split;
    const uint8_t *   qok;           // nseq + 1 entries
    uint32_t          nseq;
    uint32_t          nmin, nmax;
    const uint32_t *  uniq_pos;
    uint8_t *         mark;        // null: only write u_out / v_out
    uint32_t *        rec_u;
    uint32_t *        rec_v;
    uint32_t *        u_out;       // optional per-factor totals
    uint32_t *        v_out;
};

__global__ void k_scan_single ( uint32_t * data, uint32_t n, uint32_t * total );
// Exclusive scans (3 launches each); tile_sums holds ceil(n / kScanTile) words.
cudaError_t scan_exclusive_u8 ( const uint8_t * in, uint32_t n, uint32_t * out, uint32_t * d_total,
                                uint32_t * tile_sums, cudaStream_t st );
cudaError_t scan_exclusive_u32 ( const uint32_t * in, uint32_t n, uint32_t * out, uint32_t * d_total,
                                 uint32_t * tile_sums, cudaStream_t st );

__global__ void k_presence ( const uint8_t * raw, uint64_t total, uint32_t * present );
__global__ void k_pack ( PackArgs a );
__global__ void k_gather_key ( const uint32_t * idx, uint32_t n, const uint8_t * codes, uint32_t l, uint32_t B,
                               uint32_t lo, uint32_t * key_out );
__global__ void k_radix_hist ( const uint32_t * keys, uint32_t n, int shift, uint32_t * hist, uint32_t ntiles );
__global__ void k_radix_scatter ( const uint32_t * keys_in, const uint32_t * vals_in, uint32_t * keys_out,
                                  uint32_t * vals_out, uint32_t n, int shift, const uint32_t * offsets, uint32_t ntiles );
__global__ void k_heads ( const uint32_t * idx, const uint32_t * keys, int full_key, uint32_t n, const uint8_t * codes,
                          uint32_t l, uint8_t * head );
__global__ void k_unique ( const uint32_t * idx, const uint8_t * head, const uint32_t * pref, uint32_t n,
                           uint32_t * uniq_pos );
__global__ void k_wplanes32 ( const uint32_t * uniq_pos, uint32_t U, const uint8_t * codes, uint32_t l, uint32_t B,
                              int top_aligned, uint32_t * out );
__global__ void k_wplanes64 ( const uint32_t * uniq_pos, uint32_t U, const uint8_t * codes, uint32_t l, uint32_t B,
                              uint32_t nw64, int reversed, uint64_t * out );
__global__ void k_finalize ( FinalizeArgs a );
__global__ void k_compact ( const uint8_t * mark, const uint32_t * pref, uint32_t n, const uint32_t * rec_u,
                            const uint32_t * rec_v, uint32_t * out );

// Structured motifs, two boxes / one gap (dp_struct.cu).
struct StructArgs
{
    TextView          text;
    const uint32_t *  wpl0;          // box-0 planes of the factor ending at each position: [b * total + pos]
    const uint32_t *  wpl1;          // box-1 planes, same layout
    const uint8_t *   row_ok;        // box 0 may end at this pattern position
    const uint32_t *  row_end;       // end offset of the position's sequence
    uint32_t          total;
    uint32_t          l0, e0;        // box 0
    uint32_t          l1, e1;        // box 1 (l1 = b1)
    uint32_t          b1;
    uint32_t          gmin, gmax, G; // gap range, G = gmax - gmin + 1
    // 1, -(e0+1), -(e1+1): the Hamming kernels take a hit as the sign bit of
    // popc * one - (e+1) and shift it into their masks with multiply-adds
    // (FMA pipe; runtime values the compiler cannot fold)
    uint32_t          one, ne0, ne1;
    const ChunkInfo * chunks;
    uint32_t *        u_acc;         // [pos * G + k]
    uint32_t *        v_acc;
    uint8_t *         split_flags;   // n_split rows of total * G bytes
};

struct StructFinalizeArgs
{
    uint64_t          n;             // total * G
    const uint32_t *  u_acc;
    const uint32_t *  v_acc;
    const uint8_t *   split_flags;
    uint32_t          n_split;
    const uint8_t *   qok;
    uint32_t          nseq, nmin, nmax;
    uint8_t *         mark;
    uint32_t *        rec_u;
    uint32_t *        rec_v;
    uint32_t *        u_out;         // pair mode: totals out
    uint32_t *        v_out;
};

bool launch_dp_struct1 ( const StructArgs & a, int B, bool ed, dim3 grid, cudaStream_t st );

// Structured motifs with any number of gaps (dp_struct.cu, k_dp_structN).
constexpr uint32_t kMaxStructsN = 128;           // structures of the any-gap kernel (shared-memory counters)
constexpr uint32_t kMaxGapsN = 16;
constexpr uint32_t kStructMaxBox = 64;           // box length (and l) of structured motifs
constexpr size_t   kStructNMaxSmem = 200 * 1024; // dynamic shared memory of the any-gap kernel
struct StructNArgs
{
    TextView          text;
    const uint32_t *  wpl;           // box b's planes at [(b * B + plane) * total + pos]
    const unsigned long long * wpl64; // the same with 64-bit rows (a box longer than 32)
    bool              wide;          // rows are wpl64
    const uint8_t *   row_ok;
    const uint32_t *  row_end;       // end offset of the position's sequence
    const uint32_t *  seq_start;     // start offset of the position's sequence
    const uint32_t *  xoff;          // [k * ngaps + g]: end of box g+1 minus end of box 0, structure k
    uint32_t          total;
    uint32_t          l0, e0;
    uint32_t          blen[kMaxGapsN + 1];   // box lengths, blen[0] = l0
    uint32_t          berr[kMaxGapsN + 1];
    uint32_t          ngaps, nstructs;
    const ChunkInfo * chunks;
    uint32_t *        u_acc;         // [pos * nstructs + k]
    uint32_t *        v_acc;
    uint8_t *         split_flags;   // n_split rows of total * nstructs bytes
};
bool launch_dp_structN ( const StructNArgs & a, int B, bool ed, dim3 grid, cudaStream_t st );

/*
 * Block form of the any-gap structured search (dp_structn.cu).  A warp owns
 * Pw consecutive pattern positions and, for box g+1, the Pw + D[g] - 1 rows
 * (pattern positions P0 + lo[g] + lane) its structures reach; lane r runs
 * one row of every box, all NR = ngaps + 1 rows packed in one register.
 */
constexpr uint32_t kStructNBlkMaxRows = 4;       // boxes per structure (compiled variants: 2..4)
constexpr uint32_t kStructNBlkMaxSlots = 16;     // look-ahead ring of 32-position blocks
struct StructNBlk
{
    uint32_t Pw;                                 // pattern positions per warp
    uint32_t lo[kMaxGapsN];                      // least end offset of box g+1 over structures
    uint32_t D[kMaxGapsN];                       // distinct end offsets of box g+1
    uint32_t nslot;                              // ring slots: blocks E .. E + nslot - 1 are resident
    uint32_t lo_last;                            // lo[ngaps - 1]
    // edit distance: the rows as SWAR lanes (guard bit above each) with
    // score fields s bits below each lane's top bit
    uint32_t HB, NG, NGm1, K, SC0, s;
    uint32_t off[kStructNBlkMaxRows];            // bit offset of row b's lane
    uint32_t nm[kStructNBlkMaxRows];             // -(2^(31 - top bit of row b)): hit bit by a multiply-add
    uint32_t sd;                                 // 1: the top lane ends below bit 31 (score update by one shift)
    // Hamming: the rows as lanes of Lmax bits, factors at the top of their lanes
    uint32_t Lmax, rep;
    uint32_t hmask[kStructNBlkMaxRows];
    uint32_t ne[kStructNBlkMaxRows];             // -(e_b + 1)
    uint32_t one, two, neg1;                     // multipliers (runtime values: FMA-pipe multiply-adds)
};
// Fills *C and returns true when the shape has a block kernel (rows packable
// into one register, D <= 17, look-ahead within the ring, <= 32 structures).
bool structN_blk_shape ( const StructNArgs & a, const uint32_t * h_xoff, bool ed, StructNBlk * C );
bool launch_dp_structN_blk ( const StructNArgs & a, const StructNBlk & C, int B, bool ed, dim3 grid, cudaStream_t st );
__global__ void k_seq_start ( const uint32_t * offs, uint32_t nseq, uint64_t total, uint32_t * out );
__global__ void k_wplanes_all64 ( const uint8_t * codes, uint32_t total, uint32_t l, uint32_t B, int top_aligned,
                                  unsigned long long * out );
size_t structN_smem_bytes ( const StructNArgs & a );

// Device deduplication of passing structured entries by the writer's key
// (the boxes' symbols, gaps left out; functions.cc:1191-1239): the first
// entry of a key in print order is kept.
struct SKeyArgs
{
    const uint32_t * recs;           // 3 words per entry: pos * G + k, u, v (print order)
    uint32_t         nrec, G, NG, l;
    uint32_t         blen[kMaxGapsN];
    const uint8_t *  codes;
    const uint32_t * xoff;           // [k * NG + g]: end of box g+1 minus end of box 0
    uint32_t         tbits;          // 2^tbits table slots
    uint32_t *       rep;            // a representative entry of the slot's key (~0: empty)
    uint32_t *       first;          // least entry index with the slot's key
    uint32_t *       slot_of;        // slot of each entry
    uint8_t *        keep;
    uint32_t *       err;            // set to 1 if a probe ever visited every slot
};
__global__ void k_skey_insert ( SKeyArgs a );
__global__ void k_skey_keep ( SKeyArgs a );
__global__ void k_wplanes_all ( const uint8_t * codes, uint32_t total, uint32_t l, uint32_t B, int top_aligned,
                                uint32_t * out );
__global__ void k_struct_rows ( const uint32_t * offs, uint32_t nseq, uint64_t total, uint32_t l0, uint32_t tml,
                                uint32_t npat, uint8_t * row_ok, uint32_t * row_end );
__global__ void k_struct_finalize ( StructFinalizeArgs a );

// DP launchers (dp.cu): return false if no kernel matches the shape.
bool launch_dp_fast ( const DPArgs & a, int B, int W, int UR, bool ed, dim3 grid, cudaStream_t st );
// SWAR edit-distance lane constants (dp.cu).
struct SwarConst
{
    uint32_t HB;     // bit l-1 of every lane
    uint32_t NG;     // all bits but the guards
    uint32_t NGm1;   // NG without the lanes' top bits
    uint32_t K;      // per field 2^h - (e+1): bit h of score + K is clear exactly on a hit
    uint32_t SC0;    // per field score l
    uint32_t S;      // lane stride
    uint32_t FM;     // count field mask
    // edit distance: the hit bit h of every lane's score field, and the
    // offset of the count fields in the lanes.  NL = 2, 3: h = ceil(log2 l),
    // and the per-step count adds the hit bits where they are (count fields
    // of 6 bits at h); NL = 4 (too narrow for that): h = l-1, and the count
    // shifts the hit bits to the lane base
    uint32_t HQ, Q;
    uint32_t LIM;    // guarded-lane Hamming with three lanes: 2^(2S), the top lane's base
    uint32_t REP;    // Hamming lanes: sum of 2^(j*l), replicates an l-bit window into every lane
    // Multipliers of the edit-distance step, kernel parameters so that the
    // compiler cannot fold them: x * ONE + y, x * TWO and x * NEG1 + y run as
    // integer multiply-adds on the FMA pipe instead of adds and shifts on
    // the ALU pipe, which the logic ops already fill
    uint32_t ONE, TWO, NEG1;
};
SwarConst swar_const ( uint32_t l, uint32_t e, int NL );
// Hamming with NL = hswar_lanes(l) >= 2 factors of l bits per register
// (6 <= l <= 16, no guard bits: XOR and OR do not carry); kernels exist for
// B = 3..5 (the protein case; DNA gains nothing).
int hswar_lanes ( uint32_t l );
SwarConst hswar_const ( uint32_t l, int NL );
bool launch_dp_hswar ( const DPArgs & a, int B, int NL, int W, int UR, dim3 grid, cudaStream_t st );
// Popc-free Hamming for e <= kHclrMaxE: two factors of l bits per register in
// guarded lanes (5 <= l <= 12), or three (6 <= l <= 10, the top lane tested
// by a compare), mismatches counted by clearing each lane's lowest set bit e
// times (dp_hclr.cu); unroll 4.  hclr_lanes: the default lane count for l
// (3 where it fits), hclr_fits: whether NL lanes fit l.
constexpr uint32_t kHclrMaxE = 3;
int hclr_lanes ( uint32_t l );
bool hclr_fits ( uint32_t l, int NL );
SwarConst hclr_const ( uint32_t l, int NL );
bool launch_dp_hclr ( const DPArgs & a, int B, int NL, int W, dim3 grid, cudaStream_t st );
// Register words per thread of the packed kernels when the shape is not tuned
// (batched jobs, persistent launches, the default of an untuned job): with
// B = 4, 5 the split Eq table leaves room for enough CTAs per SM only at
// W = 4 (measured on 2000 protein sequences of 50-2000 residues, edit
// distance, k 10: W = 4 runs 352 ms, W = 8 393 ms).
__host__ __device__ constexpr int swar_default_w ( int B ) { return B >= 4 ? 4 : 8; }

// Small-job pipeline (mini.cu): one CTA per job runs every stage around the
// DP.  The host fills one MiniJob per job; result[0..2] receive the error
// flag, the distinct-factor count U and the motif count.
constexpr int kMiniThreads = 1024;
constexpr uint32_t kMiniMaxSymbols = 131072;
struct MiniJob
{
    const uint8_t *      raw;
    const uint32_t *     offs;           // nseq + 1
    const uint8_t *      qok;            // nseq + 1
    uint32_t             nseq, total, l, tml, vstart, B, nmin, nmax, n_split;
    uint32_t             nblk, plane_stride, tbits;
    int                  top_aligned;    // Hamming factor planes
    uint8_t *            codes;
    uint32_t *           planes;
    uint32_t *           vmask;
    uint32_t *           emask;
    unsigned long long * tkey;           // 2^tbits hash slots
    uint32_t *           tpos;
    uint32_t *           uniq;           // first end position of every distinct factor
    uint32_t *           wpl;            // [b * U + w]
    uint32_t *           u_acc;
    uint32_t *           v_acc;
    uint8_t *            flags;          // n_split rows of U
    uint8_t *            mark;           // total
    uint32_t *           rec_u;
    uint32_t *           rec_v;
    uint32_t *           recs;           // 3 words per motif
    uint32_t *           result;
    uint32_t *           part;           // marks per CTA share (ctas words)
    uint32_t             nwords;         // factors (bound of the distinct count)
    uint32_t             ctas;           // CTAs of this job (<= the grid's x)
    uint8_t              cmap[256];
};
constexpr uint32_t kMiniMaxCtas = 64;              // CTAs per job: one per 1024 symbols, at most this
__global__ void k_mini_clear ( const MiniJob * jobs );
__global__ void k_mini_pack ( const MiniJob * jobs );
__global__ void k_mini_uniq ( const MiniJob * jobs );
__global__ void k_mini_planes ( const MiniJob * jobs );
__global__ void k_mini_final ( const MiniJob * jobs );
__global__ void k_mini_count ( const MiniJob * jobs );
__global__ void k_mini_write ( const MiniJob * jobs );

// One job of a batched launch and one unit of its work.
struct JobDesc
{
    DPArgs    a;
    SwarConst C;
};
struct WorkItem
{
    uint32_t job, tile, chunk;
};

// Persistent batched DP over the items of one kernel class: 1-lane kernels
// (NL = 1, Hamming or edit distance) or packed ones (NL lanes; every job of
// the launch has the lane constants C).  grid = resident CTA slots.
// W register words per thread and block unroll UR: persistent_shape says
// which the persistent kernels implement (every autotuner choice for packed
// edit distance; W = 8 with the default unroll otherwise).  E >= 0: the
// popc-free Hamming form with e = E (NL 2 or 3 guarded lanes, W 8, unroll 4);
// E = -1 every other form.
bool launch_dp_persistent ( const JobDesc * jobs, const WorkItem * items, uint32_t nitems, uint32_t * counter,
                            int B, bool ed, bool scaled, int NL, int W, int UR, int E, const SwarConst & C,
                            unsigned grid, cudaStream_t st );
int persistent_ctas_per_sm ( int B, bool ed, bool scaled, int NL, int W, int UR, int E );
bool persistent_shape ( int B, bool ed, int NL, int W, int UR, int E );

// Edit distance, NL = swar_lanes(l) >= 2 factors per 32-bit register (l <= 15);
// dynamic shared memory swar_smem_bytes ( B, NL, W ).
int swar_lanes ( uint32_t l );
bool launch_dp_swar_ed ( const DPArgs & a, int B, int NL, int W, int UR, dim3 grid, cudaStream_t st );
bool launch_dp_generic ( const DPArgs & a, int B, uint32_t nw64, bool ed, dim3 grid, cudaStream_t st );

} // namespace mtx
