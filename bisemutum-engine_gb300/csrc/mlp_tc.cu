// mlp_tc.cu — the radiance cache's network on the 5th-generation tensor cores
// (tcgen05, accumulators in tensor memory): inference and the training step.
//
// A CTA of 128 threads takes 128 queries at a time; thread i owns query row i.
// Each layer is one 128 x N x 64 product, D[query][out] = sum_in
// act[query][in] W[out][in], issued as four K = 16 tcgen05.mma by one thread:
//   A  activations, 128 rows x 64 BF16 in tensor memory: lane = query row,
//      32 columns of BF16 pairs (feature 2j in the low half of column j)
//   B  the layer's weights, N rows x 64 BF16 in shared memory (N = 64, or 16
//      for the output layer: 8 weight rows and 8 zero rows)
//   D  FP32 in tensor memory: lane = query row, column = output feature.
// B is K-major with the 128-byte swizzle: a row of 64 BF16 is one 128-byte
// swizzle row, rows come in 8-row groups 1024 bytes apart, and the 16-byte
// chunk c of row r sits at chunk c ^ (r mod 8).  The K = 16 step k starts
// 32 k bytes into B's rows and 8 k columns into A.  tcgen05.commit signals an
// mbarrier when the four products are done; each warp then reads its 32 rows
// of D (tcgen05.ld 32x32b, 64 columns at once), applies ReLU and rounds to
// BF16 in one conversion per pair, and stores them (tcgen05.st, 32 columns)
// as the next layer's A.  Keeping A in tensor memory leaves shared memory
// with the weights alone: a layer moves 8 KB through it instead of 16 KB of
// stores and 24 KB of operand reads.  The weights reach shared memory by one
// bulk copy: their BF16 copies are kept in global memory in the tile layout
// (mlp_tile_index).  Rounding points (BF16 operands, FP32 accumulation) are
// those of the oracle's BF16 network; only the order of the FP32 sums differs.
//
// The training step (k_mlp_train_tc) runs forward and backward passes of
// 128-sample tiles on the same units.  The forward layers read A from tensor
// memory as inference does, and also keep each activation tile in shared
// memory, where the backward products read them in the MN-major form of the
// same swizzled tiles (no transposed copies):
//   g_a = g_z W      A: the gradient [sample][out] in tensor memory (K = out)
//                    B: W [out][in] read MN-major (N = in, K = out)
//   dW += g_z^T a    A: the gradient tile read MN-major (M = out, K = sample)
//                    B: the activation tile [sample][in] read MN-major
// The dW products are issued by a second thread and waited for two steps
// later (three gradient tiles rotate), so they run beside the chain of g_a
// products and epilogues.
// with every layer's weight gradient accumulated in tensor memory over all
// the tiles a CTA takes, and copied on its last tile (bulk copies) to the
// CTA's own FP32 gradient slot; Adam sums the slots in a fixed order.  A training CTA has 256 threads, two per sample
// row, each reading back and storing half of the row's 64 columns.
//
// Every mbarrier wait gives up after one second: the kernel then sets bit 1
// of the error word, stops issuing products and frees its tensor memory.
#include <cuda_bf16.h>
#include <atomic>
#include <cuda_runtime.h>

#include "mlp.cuh"
#include "pt_device.h"

namespace bsm {
namespace {

constexpr int kTcRows = 128;                                    // queries per tile (MMA M)
constexpr int kTcW4Rows = 16;                                   // output layer as an N = 16 product
constexpr int kTcWRows = kMlpHidden * 64 + kTcW4Rows;           // 272 weight rows in shared memory
constexpr int kTcBarOff = kTcWRows * 128;                       // 34816 = 34 x 1024
// The inference kernel's request: its 36 KB (weights, barriers, alignment slack) padded to 48 KB so that at
// most 4 CTAs share an SM, the number whose tensor memory fits (4 x 128 of 512 columns); a fifth CTA would
// wait in tcgen05.alloc until one of the four has finished all its tiles.
constexpr int kTcSmem = 48 * 1024;
static_assert(kTcBarOff + 32 + 1024 <= kTcSmem, "inference shared memory");
constexpr uint32_t kTcWBytes = (kMlpHidden * 64 + kMlpOutPad) * 128;   // 33,792: the weights' tile image
constexpr uint32_t kTcCols = 128;                               // tensor-memory columns per CTA
constexpr uint32_t kTcACol = 64;                                // first column of the A operand (32 columns)
constexpr uint32_t kTcErrTimeout = 2u;                          // error word bit: a tensor-core wait timed out

// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), BF16
// A and B (bits 7-9, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at
// bits 17-22, M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t tc_idesc(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}
// The same with A (bit 15) and / or B (bit 16) read MN-major.
__host__ __device__ constexpr uint32_t tc_idesc_mn(int m, int n, bool a_mn, bool b_mn) {
    return tc_idesc(m, n) | (a_mn ? 1u << 15 : 0u) | (b_mn ? 1u << 16 : 0u);
}

// Shared-memory matrix descriptor: start address >> 4 (bits 0-13), leading
// byte offset 16 >> 4 (bits 16-29; not used by swizzled K-major operands),
// stride byte offset 1024 >> 4 between 8-row groups (bits 32-45), descriptor
// version 1 (bits 46-47), base offset 0 (tiles are 1024-byte aligned),
// layout 2 = 128-byte swizzle (bits 61-63).
__device__ __forceinline__ uint64_t tc_sdesc(uint32_t saddr) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

// An MN-major operand in the same swizzled tiles: a tile row is one K index
// holding 64 consecutive M (or N) elements, 8-row K groups lie 1024 bytes
// apart (stride byte offset), and the leading byte offset steps to the next
// 64 M elements.  It is 0 here: an M = 128 operand reads its 64 rows twice,
// and the product's rows 64..127 repeat rows 0..63.
__device__ __forceinline__ uint64_t tc_sdesc_mn(uint32_t saddr) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)(1024 >> 4) << 32) | ((uint64_t)1 << 46) |
           ((uint64_t)2 << 61);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for the phase of parity `parity` to complete; false after one second.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    while (!mbar_try_wait(bar, parity))
        if (global_ns() - t0 > 1000000000ull) return false;
    return true;
}

// Bulk copy of `bytes` (a multiple of 16) from global to shared memory, completing on mbarrier `bar` (the
// expected byte count is announced first by the same thread).
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes become visible to the tensor core
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void tc_alloc(uint32_t slot, uint32_t cols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot), "r"(cols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tc_dealloc(uint32_t taddr, uint32_t cols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols) : "memory");
}

__device__ __forceinline__ void tc_mma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}
// The same with A read from tensor memory (`a`: its first column, lane 0).
__device__ __forceinline__ void tc_mma_ts(uint32_t d, uint32_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d),
        "r"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void tc_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// 16 columns of the warp's 32 lanes; the wait names the registers so that no
// use of them is scheduled before the load has landed.
__device__ __forceinline__ void tc_ld16(uint32_t taddr, uint32_t (&v)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(v[0]), "+r"(v[1]), "+r"(v[2]), "+r"(v[3]), "+r"(v[4]), "+r"(v[5]), "+r"(v[6]), "+r"(v[7]),
                   "+r"(v[8]), "+r"(v[9]), "+r"(v[10]), "+r"(v[11]), "+r"(v[12]), "+r"(v[13]), "+r"(v[14]),
                   "+r"(v[15])
                 :
                 : "memory");
}

// 32 columns in one load and one wait.
__device__ __forceinline__ void tc_ld32(uint32_t taddr, uint32_t (&v)[32]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {"
                 "%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                 "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31"
                 "}, [%32];"
                 : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                   "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
                   "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
                   "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
                 : "r"(taddr)
                 : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(v[0]), "+r"(v[1]), "+r"(v[2]), "+r"(v[3]), "+r"(v[4]), "+r"(v[5]), "+r"(v[6]), "+r"(v[7]),
                   "+r"(v[8]), "+r"(v[9]), "+r"(v[10]), "+r"(v[11]), "+r"(v[12]), "+r"(v[13]), "+r"(v[14]), "+r"(v[15]),
                   "+r"(v[16]), "+r"(v[17]), "+r"(v[18]), "+r"(v[19]), "+r"(v[20]), "+r"(v[21]), "+r"(v[22]), "+r"(v[23]),
                   "+r"(v[24]), "+r"(v[25]), "+r"(v[26]), "+r"(v[27]), "+r"(v[28]), "+r"(v[29]), "+r"(v[30]), "+r"(v[31])
                 :
                 : "memory");
}

// 64 columns in one load and one wait.
__device__ __forceinline__ void tc_ld64(uint32_t taddr, uint32_t (&v)[64]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x64.b32 {"
                 "%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                 "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,"
                 "%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47,"
                 "%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63"
                 "}, [%64];"
                 : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                   "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
                   "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
                   "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31]),
                   "=r"(v[32]), "=r"(v[33]), "=r"(v[34]), "=r"(v[35]), "=r"(v[36]), "=r"(v[37]), "=r"(v[38]), "=r"(v[39]),
                   "=r"(v[40]), "=r"(v[41]), "=r"(v[42]), "=r"(v[43]), "=r"(v[44]), "=r"(v[45]), "=r"(v[46]), "=r"(v[47]),
                   "=r"(v[48]), "=r"(v[49]), "=r"(v[50]), "=r"(v[51]), "=r"(v[52]), "=r"(v[53]), "=r"(v[54]), "=r"(v[55]),
                   "=r"(v[56]), "=r"(v[57]), "=r"(v[58]), "=r"(v[59]), "=r"(v[60]), "=r"(v[61]), "=r"(v[62]), "=r"(v[63])
                 : "r"(taddr)
                 : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(v[0]), "+r"(v[1]), "+r"(v[2]), "+r"(v[3]), "+r"(v[4]), "+r"(v[5]), "+r"(v[6]), "+r"(v[7]),
                   "+r"(v[8]), "+r"(v[9]), "+r"(v[10]), "+r"(v[11]), "+r"(v[12]), "+r"(v[13]), "+r"(v[14]), "+r"(v[15]),
                   "+r"(v[16]), "+r"(v[17]), "+r"(v[18]), "+r"(v[19]), "+r"(v[20]), "+r"(v[21]), "+r"(v[22]), "+r"(v[23]),
                   "+r"(v[24]), "+r"(v[25]), "+r"(v[26]), "+r"(v[27]), "+r"(v[28]), "+r"(v[29]), "+r"(v[30]), "+r"(v[31]),
                   "+r"(v[32]), "+r"(v[33]), "+r"(v[34]), "+r"(v[35]), "+r"(v[36]), "+r"(v[37]), "+r"(v[38]), "+r"(v[39]),
                   "+r"(v[40]), "+r"(v[41]), "+r"(v[42]), "+r"(v[43]), "+r"(v[44]), "+r"(v[45]), "+r"(v[46]), "+r"(v[47]),
                   "+r"(v[48]), "+r"(v[49]), "+r"(v[50]), "+r"(v[51]), "+r"(v[52]), "+r"(v[53]), "+r"(v[54]), "+r"(v[55]),
                   "+r"(v[56]), "+r"(v[57]), "+r"(v[58]), "+r"(v[59]), "+r"(v[60]), "+r"(v[61]), "+r"(v[62]), "+r"(v[63])
                 :
                 : "memory");
}

// 32 columns of the warp's 32 lanes stored, then waited for (the stores complete before the thread goes on).
__device__ __forceinline__ void tc_st32(uint32_t taddr, const uint32_t (&v)[32]) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {"
                 "%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,"
                 "%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32"
                 "};" ::"r"(taddr),
                 "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]),
                 "r"(v[8]), "r"(v[9]), "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]), "r"(v[15]),
                 "r"(v[16]), "r"(v[17]), "r"(v[18]), "r"(v[19]), "r"(v[20]), "r"(v[21]), "r"(v[22]), "r"(v[23]),
                 "r"(v[24]), "r"(v[25]), "r"(v[26]), "r"(v[27]), "r"(v[28]), "r"(v[29]), "r"(v[30]), "r"(v[31])
                 : "memory");
    asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

// 16 and 8 columns of the warp's 32 lanes stored, then waited for.
__device__ __forceinline__ void tc_st16(uint32_t taddr, const uint32_t (&v)[16]) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {"
                 "%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(taddr),
                 "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]),
                 "r"(v[8]), "r"(v[9]), "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]), "r"(v[15])
                 : "memory");
    asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tc_st8(uint32_t taddr, const uint32_t (&v)[8]) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(taddr),
                 "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7])
                 : "memory");
    asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}

// max(lo, 0) and max(hi, 0) rounded to BF16 in one conversion (cvt.rn.relu); lo in the low half.
__device__ __forceinline__ uint32_t pack2_relu(float lo, float hi) {
    uint32_t r;
    asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
    return r;
}

// 16-byte chunk c (features 8c..8c+7) of row r of a swizzled 128-row tile.
__device__ __forceinline__ uint4* tile_chunk(unsigned char* tile, int r, int c) {
    return reinterpret_cast<uint4*>(tile + r * 128 + ((c ^ (r & 7)) << 4));
}

// The weights into rows 0..271 of the tile at `base`: rows 0..263 by one bulk copy of their tile image (the
// BF16 copies are kept in that layout, mlp_tile_index), completing on `wbar`; rows 264..271 zeroed.  Thread 0
// starts the copy; every thread waits on `wbar` (phase 0) before the first product reads the tile.
__device__ __forceinline__ void load_weights_async(const __nv_bfloat16* w, unsigned char* base, uint32_t base_s,
                                                   uint32_t wbar, int tid) {
    if (tid == 0) {
        mbar_init(wbar, 1);
        mbar_expect_tx(wbar, kTcWBytes);
        bulk_load(base_s, w, kTcWBytes, wbar);
    }
    if (tid < 64) *tile_chunk(base, kMlpHidden * 64 + kMlpOutPad + (tid >> 3), tid & 7) = make_uint4(0u, 0u, 0u, 0u);
}

// Encoded features of one query (the encoding of mlp_feature) as 32 BF16
// pairs, feature 2j in the low half of word j: words 4d..4d+3 (d < 7) hold
// sin/cos(2^k pi raw[d]), k = 0..3; words 28..31 hold raw[7..11], 1, 0, 0.
// The base frequency comes from
// the special-function unit (__sincosf: absolute error below 2^-21 for
// arguments in [-pi, pi], which pi raw[d] is for the normalised inputs);
// frequencies k > 0 come from k - 1 by the double-angle identities
// (sin 2a = 2 sin a cos a, cos 2a = (cos a - sin a)(cos a + sin a)).  Both
// errors lie far below the BF16 rounding that follows; the training and the
// inference kernels share this encoding.
__device__ __forceinline__ void encode_words(const float (&raw)[kMlpRaw], uint32_t (&p)[32]) {
#pragma unroll
    for (int d = 0; d < 7; ++d) {
        float s, c;
        __sincosf(raw[d] * 3.14159265f, &s, &c);
        p[4 * d] = pack2(s, c);
#pragma unroll
        for (int k = 1; k < 4; ++k) {
            float s2 = 2.0f * s * c, c2 = (c - s) * (c + s);
            s = s2;
            c = c2;
            p[4 * d + k] = pack2(s, c);
        }
    }
    p[28] = pack2(raw[7], raw[8]);
    p[29] = pack2(raw[9], raw[10]);
    p[30] = pack2(raw[11], 1.0f);
    p[31] = pack2(0.0f, 0.0f);
}

// kInfer: queries (4 float4: raw[0..11], then throughput rgb and the pixel
// accumulator index bits), n = min(*count, n_max); adds throughput x max(y, 0)
// to the accumulator (to the fixed-point sums `accum_fx` when set).  Otherwise: samples (raw in the first 3 float4), n =
// n_max, writes y (3 floats per sample) to out.
template <bool kInfer>
__global__ void __launch_bounds__(kTcRows) k_mlp_forward_tc(const __nv_bfloat16* __restrict__ w,
                                                            const float4* __restrict__ q, const uint32_t* count,
                                                            uint32_t n_max, float4* accum,
                                                            unsigned long long* accum_fx, float* out, uint32_t* err) {
    extern __shared__ unsigned char smem_raw[];
    const uint32_t raw_s = smem_u32(smem_raw);
    const uint32_t base_s = (raw_s + 1023u) & ~1023u;
    unsigned char* base = smem_raw + (base_s - raw_s);
    const uint32_t bar = base_s + kTcBarOff;
    const uint32_t wbar = bar + 8;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(base + kTcBarOff + 16);
    const int tid = threadIdx.x, warp = tid >> 5;

    const uint32_t n = kInfer ? min(*count, n_max) : n_max;
    const bool has_work = blockIdx.x * kTcRows < n;   // CTAs past the queries copy no weights
    if (has_work) load_weights_async(w, base, base_s, wbar, tid);
    if (tid == 0) mbar_init(bar, 1);
    __syncwarp();
    if (warp == 0) tc_alloc(smem_u32(tmem_slot), kTcCols);
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t rows_tmem = tmem + ((uint32_t)(warp * 32) << 16);   // this warp's 32 lanes
    uint32_t phase = 0;
    bool failed = false;

    // this row's query of the next tile, loaded while the current tile is in the tensor cores
    auto fetch = [&](uint32_t row, float4 (&f)[4]) {
#pragma unroll
        for (int k = 0; k < 4; ++k)
            f[k] = row < n && (kInfer || k < 3) ? q[4 * (size_t)row + k] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    };
    float4 next[4];
    fetch(blockIdx.x * kTcRows + tid, next);
    bool weights = false;   // the weight copy has landed
    for (uint32_t tile = blockIdx.x; tile * kTcRows < n && !failed; tile += gridDim.x) {
        const uint32_t row = tile * kTcRows + tid;
        const float4 m = next[3];   // throughput and accumulator index (queries)
        {
            float raw[kMlpRaw];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                raw[4 * k] = next[k].x; raw[4 * k + 1] = next[k].y; raw[4 * k + 2] = next[k].z; raw[4 * k + 3] = next[k].w;
            }
            fetch(row + gridDim.x * kTcRows, next);
            uint32_t p[32];
            encode_words(raw, p);
            tc_st32(rows_tmem + kTcACol, p);
        }
        const bool w_ok = weights || mbar_wait(wbar, 0);
        weights = true;
        fence_async_smem();   // the zeroed weight rows
        tc_fence_before();
        if (__syncthreads_or(!w_ok)) { failed = true; break; }
        for (int l = 0; l <= kMlpHidden; ++l) {
            if (tid == 0) {
                tc_fence_after();
                const uint32_t w_s = base_s + l * 64 * 128;
                const uint32_t idesc = l < kMlpHidden ? tc_idesc(kTcRows, 64) : tc_idesc(kTcRows, kTcW4Rows);
#pragma unroll
                for (int k = 0; k < 4; ++k) tc_mma_ts(tmem, tmem + kTcACol + 8 * k, tc_sdesc(w_s + 32 * k), idesc, k);
                tc_commit(bar);
            }
            __syncwarp();
            const bool done = mbar_wait(bar, phase);
            phase ^= 1u;
            __syncwarp();   // the tensor-memory loads below are warp-collective
            tc_fence_after();
            if (l < kMlpHidden) {
                uint32_t v[64], p[32];
                tc_ld64(rows_tmem, v);
#pragma unroll
                for (int i = 0; i < 32; ++i) p[i] = pack2_relu(__uint_as_float(v[2 * i]), __uint_as_float(v[2 * i + 1]));
                tc_st32(rows_tmem + kTcACol, p);   // the next layer's A
            } else {
                uint32_t v[16];
                tc_ld16(rows_tmem, v);
                float y0 = __uint_as_float(v[0]), y1 = __uint_as_float(v[1]), y2 = __uint_as_float(v[2]);
                if (done && row < n) {
                    if (kInfer) {
                        const float c0 = m.x * fmaxf(y0, 0.0f), c1 = m.y * fmaxf(y1, 0.0f), c2 = m.z * fmaxf(y2, 0.0f);
                        if (accum_fx) accum_fixed_add(accum_fx, __float_as_uint(m.w), c0, c1, c2);
                        else atomicAdd(accum + __float_as_uint(m.w), make_float4(c0, c1, c2, 0.0f));
                    } else {
                        out[3 * (size_t)row] = y0;
                        out[3 * (size_t)row + 1] = y1;
                        out[3 * (size_t)row + 2] = y2;
                    }
                }
            }
            tc_fence_before();
            if (__syncthreads_or(!done)) { failed = true; break; }
        }
    }
    if (failed) {
        if (tid == 0) {
            atomicOr(err, kTcErrTimeout);
            mbar_wait(bar, phase ^ 1u);   // the products of the abandoned layer, once more bounded
        }
        tc_fence_before();
    }
    if (has_work && !weights && tid == 0) mbar_wait(wbar, 0);   // no copy into shared memory outlives the CTA
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tc_dealloc(tmem, kTcCols);
    }
}

// ------------------------------------------------------------- training ----
// Shared memory of k_mlp_train_tc: the weights (as the forward kernel), the
// five activation tiles of a 128-sample tile (encoded input e, a0..a3), three
// gradient tiles that rotate over the backward steps (gy, gz3, gz2, gz1, gz0:
// a step's weight-gradient product may still read its tile while the next two
// steps run), the mbarriers and the tensor-memory address (183 KB: one CTA per SM).
constexpr int kTrTile = kTcRows * 128;                          // 16 KB per 128 x 64 BF16 tile
constexpr int kTrActOff = kTcWRows * 128;                       // 34816
constexpr int kTrGradOff = kTrActOff + 5 * kTrTile;             // 116736
constexpr int kTrBarOff = kTrGradOff + 3 * kTrTile;             // 165888
// 16 KB beyond the barrier are never written: every operand window of the products
// (start + 16 rows x 128 bytes per K step, or a whole 16 KB tile read K-major)
// lies inside the allocation.
constexpr int kTrSmem = kTrBarOff + 16384 + 1024;
// Tensor memory: columns 0..63 hold the product being read back (forward z,
// backward g_a); 64 + 64 l .. 127 + 64 l hold dW_l (l = 0..4; rows = outputs);
// 384..415 hold the A operand (activations, then gradients) as BF16 pairs.
constexpr uint32_t kTrCols = 512;
constexpr int kTrThreads = 256;                                 // two threads per sample row
constexpr uint32_t kTrDw = 64;
constexpr uint32_t kTrA = kTrDw + 5 * 64;                       // 384: the A operand (32 columns)
static_assert(kTrGradOff % 1024 == 0 && kTrBarOff % 1024 == 0, "swizzled tiles start on 1024-byte boundaries");
static_assert(kTrA + 32 <= kTrCols, "tensor-memory columns");

// Bulk copy of `bytes` (a multiple of 16) from shared to global memory, tracked by this thread's bulk-async
// group.
__device__ __forceinline__ void bulk_store(void* gdst, uint32_t ssrc, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(gdst), "r"(ssrc), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_wait_all() {
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
    asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

// g_z = g_a * (a > 0) for this thread's 32 columns v of its row of g_a, as 16 BF16 pairs (a: the same
// columns of the activation row, 4 chunks).
__device__ __forceinline__ void relu_grad_words(const uint32_t (&v)[32], const uint4 (&a)[4], uint32_t (&p)[16]) {
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const uint32_t av[4] = {a[c].x, a[c].y, a[c].z, a[c].w};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int j = 4 * c + i;
            const float lo = __uint_as_float(av[i] << 16) > 0.0f ? __uint_as_float(v[2 * j]) : 0.0f;
            const float hi = __uint_as_float(av[i] & 0xffff0000u) > 0.0f ? __uint_as_float(v[2 * j + 1]) : 0.0f;
            p[j] = pack2(lo, hi);
        }
    }
}

// Half h of the encoded features of one sample (features 32 h .. 32 h + 31) as 16 BF16 pairs, word 4 d + k
// of chunk 4 h + d: h = 0 encodes raw[0..3] (f0) as chunks 0..3; h = 1 encodes raw[4..6] (f0.xyz) as chunks
// 4..6 and fills chunk 7 from raw[7] = f0.w and raw[8..11] = f1.  The values are those of encode_words.
__device__ __forceinline__ void encode_half(int h, const float4& f0, const float4& f1, uint32_t (&p)[16]) {
    const float x[4] = {f0.x, f0.y, f0.z, f0.w};
#pragma unroll
    for (int d = 0; d < 4; ++d) {
        if (h && d == 3) break;
        float s, c;
        __sincosf(x[d] * 3.14159265f, &s, &c);
        p[4 * d] = pack2(s, c);
#pragma unroll
        for (int k = 1; k < 4; ++k) {
            float s2 = 2.0f * s * c, c2 = (c - s) * (c + s);
            s = s2;
            c = c2;
            p[4 * d + k] = pack2(s, c);
        }
    }
    if (h) {
        p[12] = pack2(f0.w, f1.x);
        p[13] = pack2(f1.y, f1.z);
        p[14] = pack2(f1.w, 1.0f);
        p[15] = pack2(0.0f, 0.0f);
    }
}

// Row r's words p (16 per half h, as encode_half lays them out) into the chunks 4 h .. 4 h + 3 of a tile.
__device__ __forceinline__ void store_half(unsigned char* tile, int r, int h, const uint32_t (&p)[16]) {
#pragma unroll
    for (int c = 0; c < 4; ++c) *tile_chunk(tile, r, 4 * h + c) = make_uint4(p[4 * c], p[4 * c + 1], p[4 * c + 2], p[4 * c + 3]);
}

// r[j] = v[(j + k) mod 4] for k = 0..3 in two conditional rotations (no indexed register access).
__device__ __forceinline__ void rotate4(uint4 (&r)[4], uint32_t k) {
#pragma unroll
    for (int b = 0; b < 2; ++b) {
        const int sh = 1 << b;
        const bool on = (k >> b) & 1u;
        uint4 t[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) t[j] = on ? r[(j + sh) & 3] : r[j];
#pragma unroll
        for (int j = 0; j < 4; ++j) r[j] = t[j];
    }
}

// One layer's weight gradient from tensor memory into shared memory as FP32 [out][64] (rows < `rows`), by all
// eight warps: warp w reads its lanes (lane o = output o; lanes 64..127 repeat 0..63), rows 32 (w & 1) + lane,
// columns 16 (w >> 1) .. 16 (w >> 1) + 15.  Lanes store their four 16-byte chunks rotated by the lane index.
__device__ __forceinline__ void stage_weight_grad(uint32_t dw, uint32_t rows, float* stage, int warp, int lane) {
    const uint32_t o = (uint32_t)((warp & 1) * 32 + lane);
    const uint32_t c0 = 16u * (uint32_t)(warp >> 1);
    uint32_t v[16];
    tc_ld16(dw + c0, v);
    if (o < rows) {
        uint4 r[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) r[i] = make_uint4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
        const uint32_t k = (uint32_t)lane & 3u;
        rotate4(r, k);
        float* row = stage + o * 64 + c0;
#pragma unroll
        for (int j = 0; j < 4; ++j) *reinterpret_cast<uint4*>(row + 4 * ((j + k) & 3u)) = r[j];
    }
}

// samples: 4 float4 each (raw inputs in the first three, the target rgb in
// the fourth).  Writes the CTA's share of the gradient of the mean relative
// L2 loss over the n samples, sum over channels of (y - t)^2 / (y^2 + 0.01) /
// (3 n) with the denominator held constant, to its slot dW_parts + CTA x
// kMlpParams (summed over the slots in a fixed order afterwards, so the
// gradient does not depend on which CTA finishes first), and adds the loss to
// loss_out[0].
// Rounding points: encoded inputs, activations and gradients g_y, g_z in
// BF16, products in FP32 (those of the oracle's BF16 network).
//
// 256 threads: threads t and t + 128 share sample row t of the tile.  The
// first (warps 0..3) loads the sample's raw inputs 0..3 and its target,
// encodes features 0..31, and reads back columns 0..31 of every product;
// the second (warps 4..7, which reach the same tensor-memory lanes) loads
// raw inputs 4..11 and takes features and columns 32..63.
__global__ void __launch_bounds__(kTrThreads, 1) k_mlp_train_tc(const __nv_bfloat16* __restrict__ w,
                                                                const float4* __restrict__ s, uint32_t n,
                                                                float* dW_parts, float* loss_out, uint32_t* err) {
    extern __shared__ unsigned char smem_raw[];
    const uint32_t raw_s = smem_u32(smem_raw);
    const uint32_t base_s = (raw_s + 1023u) & ~1023u;
    unsigned char* base = smem_raw + (base_s - raw_s);
    const uint32_t act_s = base_s + kTrActOff, grad_s = base_s + kTrGradOff, bar = base_s + kTrBarOff;
    unsigned char* act = base + kTrActOff;
    unsigned char* grad = base + kTrGradOff;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(base + kTrBarOff + 8);
    const uint32_t wbar = bar + 16;
    // the weight-gradient products (issued by thread 128): dW_L commits to dwbar(L & 1), so that each barrier
    // has at most one commit outstanding when it is waited on (the waits lag the commits by two steps)
    auto dwbar = [&](int L) -> uint32_t { return bar + 24 + 8 * (uint32_t)(L & 1); };
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, r = tid & (kTcRows - 1), h = tid >> 7;

    // this thread's half of its row's sample in the next tile, loaded ahead: the first before the weights
    float4 nx[2];
    auto fetch = [&](uint32_t row) {
        nx[0] = row < n ? s[4 * (size_t)row + (h ? 1 : 0)] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        nx[1] = row < n ? s[4 * (size_t)row + (h ? 2 : 3)] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    };
    fetch(blockIdx.x * kTcRows + r);
    load_weights_async(w, base, base_s, wbar, tid);
    if (tid == 0) {
        mbar_init(bar, 1);
        mbar_init(dwbar(0), 1);
        mbar_init(dwbar(1), 1);
    }
    __syncwarp();
    if (warp == 0) tc_alloc(smem_u32(tmem_slot), kTrCols);
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t rows_tmem = tmem + ((uint32_t)((warp & 3) * 32) << 16);   // this warp's 32 lanes
    const uint32_t cols = 32u * (uint32_t)h;                                  // this thread's 32 columns
    const uint32_t a_half = rows_tmem + kTrA + 16u * (uint32_t)h;             // its 16 columns of A
    const float inv = 1.0f / (3.0f * (float)n);
    float loss = 0.0f;
    uint32_t phase = 0, dw_phase[2] = {0u, 0u};
    bool failed = false;
    const uint32_t tiles = (n + kTcRows - 1) / kTcRows;

    // all threads wait for the products committed to `b`; false when the wait timed out
    auto wait_products = [&](uint32_t b, uint32_t& ph) -> bool {
        __syncwarp();
        const bool ok = mbar_wait(b, ph);
        ph ^= 1u;
        __syncwarp();
        tc_fence_after();
        return ok;
    };
    // dW_L is complete after stage L of the CTA's last tile, and act tile L is no longer read: all threads stage
    // it there, and thread 0 copies it to the CTA's gradient slot with a bulk copy that overlaps the remaining work
    float* const dW_slot = dW_parts + (size_t)blockIdx.x * kMlpParams;
    auto reduce_weight_grad = [&](int L) {
        tc_fence_after();
        const uint32_t rows = L < kMlpHidden ? 64u : (uint32_t)kMlpOut;
        stage_weight_grad(rows_tmem + kTrDw + 64 * (uint32_t)L, rows, reinterpret_cast<float*>(act + L * kTrTile),
                          warp, lane);
        tc_fence_before();
        fence_async_smem();
        __syncthreads();
        if (tid == 0) bulk_store(dW_slot + L * kMlpLayerParams, act_s + L * kTrTile, rows * 64u * 4u);
    };
    // all threads' shared- and tensor-memory writes reach the tensor core; true when some thread's wait timed out
    auto publish = [&](bool done) -> bool {
        fence_async_smem();
        tc_fence_before();
        return __syncthreads_or(!done) != 0;
    };

    // Products: the forward layers and the backward g_a read A (activations, then gradients) from tensor
    // memory (columns kTrA..), where each thread stores its 16 columns, and B (the weights) from shared
    // memory; the weight gradients dW_L += g_in^T a(L-1) read both operands from the shared-memory tiles
    // (MN-major), issued by thread 128 and waited for two steps later, so that they run while the chain of
    // g_a products and their epilogues goes on.  The gradient of step L lives in tile gtile(L).
    auto gtile = [](int L) -> uint32_t { return (uint32_t)((kMlpHidden - L) % 3) * kTrTile; };
    auto wait_dw = [&](int L) -> bool { return wait_products(dwbar(L), dw_phase[L & 1]); };
    for (uint32_t tile = blockIdx.x; tile < tiles && !failed; tile += gridDim.x) {
        const bool first = tile == blockIdx.x, last = tile + gridDim.x >= tiles;
        const uint32_t row = tile * kTcRows + r;
        const float4 f0 = nx[0], f1 = nx[1];   // h = 0: f1 is the target
        fetch(row + gridDim.x * kTcRows);
        {
            uint32_t p[16];
            encode_half(h, f0, f1, p);
            store_half(act, r, h, p);   // e, read by dW_0
            tc_st16(a_half, p);         // A of layer 0
        }
        if (publish(!first || mbar_wait(wbar, 0))) { failed = true; break; }
        // forward: act[l + 1] = relu(act[l] W_l^T), y = a3 W4^T
        float y0 = 0.0f, y1 = 0.0f, y2 = 0.0f;
        for (int l = 0; l <= kMlpHidden && !failed; ++l) {
            if (tid == 0) {
                tc_fence_after();
                const uint32_t w_s = base_s + l * 64 * 128;
                const uint32_t idesc = l < kMlpHidden ? tc_idesc(kTcRows, 64) : tc_idesc(kTcRows, kTcW4Rows);
#pragma unroll
                for (int k = 0; k < 4; ++k) tc_mma_ts(tmem, tmem + kTrA + 8 * k, tc_sdesc(w_s + 32 * k), idesc, k);
                tc_commit(bar);
            }
            const bool done = wait_products(bar, phase);
            if (l < kMlpHidden) {
                uint32_t v[32], p[16];
                tc_ld32(rows_tmem + cols, v);
#pragma unroll
                for (int i = 0; i < 16; ++i) p[i] = pack2_relu(__uint_as_float(v[2 * i]), __uint_as_float(v[2 * i + 1]));
                store_half(act + (l + 1) * kTrTile, r, h, p);   // a_l, read by the backward pass
                tc_st16(a_half, p);                              // A of layer l + 1
            } else if (h == 0) {
                uint32_t v[16];
                tc_ld16(rows_tmem, v);
                y0 = __uint_as_float(v[0]); y1 = __uint_as_float(v[1]); y2 = __uint_as_float(v[2]);
            }
            if (publish(done)) failed = true;
        }
        if (failed) break;
        // loss gradient g_y (rows >= n: zero): gradient tile 0 (chunk 0: channels 0..7; the rest zero) and, as
        // the A of g_a(4) (K = 16), tensor-memory columns kTrA .. kTrA + 7
        if (h == 0) {
            const float yv[3] = {y0, y1, y2}, tv[3] = {f1.x, f1.y, f1.z};
            float gy[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float d = yv[c] - tv[c], rden = __frcp_rn(yv[c] * yv[c] + 0.01f) * inv;
                loss += row < n ? d * d * rden : 0.0f;
                gy[c] = row < n ? 2.0f * d * rden : 0.0f;
            }
            const uint32_t g[8] = {pack2(gy[0], gy[1]), pack2(gy[2], 0.0f), 0u, 0u, 0u, 0u, 0u, 0u};
            *tile_chunk(grad, r, 0) = make_uint4(g[0], g[1], 0u, 0u);
            tc_st8(rows_tmem + kTrA, g);
        }
#pragma unroll
        for (int c = 0; c < 4; ++c)
            if (h || c > 0) *tile_chunk(grad, r, 4 * h + c) = make_uint4(0u, 0u, 0u, 0u);
        if (publish(true)) { failed = true; break; }
        // backward: step L reads gradient tile gtile(L) (g_y, then g_z3 .. g_z0; the same values as A in tensor
        // memory), adds dW_L and, for L > 0, writes g_z(L-1) = (g_in W_L) * (a(L-1) > 0) into tile gtile(L-1)
        // and into A
        for (int L = kMlpHidden; L >= 0 && !failed; --L) {
            const uint32_t g_s = grad_s + gtile(L);
            const uint32_t a_s = act_s + L * kTrTile;   // a(L-1): e for L = 0, a3 for L = 4
            uint4 ar[4];                                  // this thread's half of the mask row: a(L-1) > 0
            if (L > 0)
#pragma unroll
                for (int c = 0; c < 4; ++c) ar[c] = *tile_chunk(act + L * kTrTile, r, 4 * h + c);
            // dW_{L+2} has read tile gtile(L-1) = gtile(L+2), which this step overwrites, and is in tensor memory
            bool done = L + 2 > kMlpHidden || wait_dw(L + 2);
            if (tid == 0 && L > 0) {   // g_a = g_in W_L: K = outputs of layer L (16 for the output layer)
                tc_fence_after();
                const uint32_t w_s = base_s + L * 64 * 128;
                const uint32_t idesc = tc_idesc_mn(kTcRows, 64, false, true);
                const int ks = L == kMlpHidden ? 1 : 4;
                for (int k = 0; k < ks; ++k) tc_mma_ts(tmem, tmem + kTrA + 8 * k, tc_sdesc_mn(w_s + 2048 * k), idesc, k);
                tc_commit(bar);
            }
            if (tid == 128) {   // dW_L += g_in^T a(L-1): M = outputs (rows 64..127 repeat them), K = the 128 samples
                tc_fence_after();
                const uint32_t idesc = tc_idesc_mn(kTcRows, 64, true, true);
                const uint32_t d = tmem + kTrDw + 64 * (uint32_t)L;
#pragma unroll
                for (int k = 0; k < kTcRows / 16; ++k)
                    tc_mma(d, tc_sdesc_mn(g_s + 2048 * k), tc_sdesc_mn(a_s + 2048 * k), idesc, first && k == 0 ? 0u : 1u);
                tc_commit(dwbar(L));
            }
            // the layer two steps back, complete on the last tile, while this step's products run
            if (last && L + 2 <= kMlpHidden) reduce_weight_grad(L + 2);
            if (L > 0) {
                done = wait_products(bar, phase) && done;
                uint32_t v[32], p[16];
                tc_ld32(rows_tmem + cols, v);
                relu_grad_words(v, ar, p);
                store_half(grad + gtile(L - 1), r, h, p);   // read by dW_(L-1)
                tc_st16(a_half, p);                         // A of g_a(L-1)
            }
            if (publish(done)) failed = true;
        }
        // dW_1 and dW_0: the next tile's forward pass overwrites the tiles they read
        if (!failed && publish(wait_dw(1) && wait_dw(0))) failed = true;
        if (last && !failed) reduce_weight_grad(1);
        if (last && !failed) reduce_weight_grad(0);
    }
    // loss: one atomic per warp
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, off);
    if (lane == 0 && loss != 0.0f) atomicAdd(loss_out, loss);
    if (failed) {
        if (tid == 0) {
            atomicOr(err, kTcErrTimeout);
            mbar_wait(bar, phase ^ 1u);     // the products of the abandoned round, once more bounded
            mbar_wait(dwbar(0), dw_phase[0] ^ 1u);
            mbar_wait(dwbar(1), dw_phase[1] ^ 1u);
        }
        tc_fence_before();
    }
    if (tid == 0) bulk_wait_all();   // the weight-gradient copies (shared memory is read until they end)
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tc_dealloc(tmem, kTrCols);
    }
}

// Per device (ordinal < 64): the opt-in shared-memory size is a per-device function attribute.
std::atomic<uint64_t> g_tc_attr{0};
int g_tc_grid[64] = {};

cudaError_t tc_setup(int device) {
    if (device < 0 || device >= 64) return cudaErrorInvalidDevice;
    if (!(g_tc_attr.load() & (1ull << device))) {
        cudaError_t e = cudaFuncSetAttribute(k_mlp_forward_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_mlp_forward_tc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_mlp_train_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kTrSmem);
        if (e != cudaSuccess) return e;
        g_tc_attr.fetch_or(1ull << device);
    }
    if (!g_tc_grid[device]) {
        int sms = 0;
        cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
        if (e != cudaSuccess) return e;
        g_tc_grid[device] = sms * 4;   // 4 CTAs per SM: 4 x 128 of 512 tensor-memory columns
    }
    return cudaSuccess;
}

}  // namespace

cudaError_t launch_mlp_infer(int device, cudaStream_t st, const void* wb, const float4* queries, const uint32_t* count,
                             uint32_t capacity, float4* accum, unsigned long long* accum_fx, uint32_t* err) {
    cudaError_t e = tc_setup(device);
    if (e != cudaSuccess) return e;
    k_mlp_forward_tc<true><<<g_tc_grid[device], kTcRows, kTcSmem, st>>>((const __nv_bfloat16*)wb, queries, count, capacity,
                                                                accum, accum_fx, nullptr, err);
    return cudaGetLastError();
}

cudaError_t launch_mlp_train(int device, cudaStream_t st, const void* wb, const float4* samples, uint32_t n,
                             float* dW_parts, uint32_t* parts, float* loss, uint32_t* err) {
    *parts = 0;
    cudaError_t e = tc_setup(device);
    if (e != cudaSuccess) return e;
    if (n == 0) return cudaSuccess;
    // one CTA per SM (512 tensor-memory columns, 183 KB of shared memory), 128 samples at a time
    const uint32_t tiles = (n + kTcRows - 1) / kTcRows, sms = (uint32_t)g_tc_grid[device] / 4;
    *parts = tiles < sms ? tiles : sms;
    k_mlp_train_tc<<<*parts, kTrThreads, kTrSmem, st>>>((const __nv_bfloat16*)wb, samples, n, dW_parts, loss, err);
    return cudaGetLastError();
}

uint32_t mlp_train_parts(int device) { return tc_setup(device) == cudaSuccess ? (uint32_t)g_tc_grid[device] / 4 : 0u; }

cudaError_t launch_mlp_predict(int device, cudaStream_t st, const void* wb, const float4* samples, uint32_t n,
                               float* out, uint32_t* err) {
    cudaError_t e = tc_setup(device);
    if (e != cudaSuccess) return e;
    if (n == 0) return cudaSuccess;
    uint32_t tiles = (n + kTcRows - 1) / kTcRows;
    uint32_t grid = tiles < (uint32_t)g_tc_grid[device] ? tiles : (uint32_t)g_tc_grid[device];
    k_mlp_forward_tc<false><<<grid, kTcRows, kTcSmem, st>>>((const __nv_bfloat16*)wb, samples, nullptr, n, nullptr,
                                                            nullptr, out, err);
    return cudaGetLastError();
}

}  // namespace bsm
