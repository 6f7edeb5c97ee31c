// gs_oracle_wgpusort.cpp — CPU oracle (test infrastructure only): a literal serial re-execution of
// the reference's radix sorter, the wgpu_sort port behind RadixSorter::sort / sort_indirect
// (src/radix_sorter.rs:56-96, 600-669; kernels src/shader/radix_sort.wgsl:78-529), as the crate
// builds it: subgroup size 1 (src/radix_sorter.rs:73), 8-bit digits, 4 passes, blocks of
// 256 x 15 = 3840 keys (src/radix_sorter.rs:150-178), the sorter state's num_keys = N
// (src/radix_sorter.rs:485-492) and an indirect dispatch of x = ceil(V / 3840) workgroups written
// by the preprocess `post` (src/shader/preprocess.wesl:108-126).
//
// Every workgroup's steps are restated in the shader's order: zero_histograms, calculate_histogram,
// prefix_histogram (a Blelloch scan), then scatter_even / scatter_odd / scatter_even / scatter_odd
// with their partition status encodings (even: invalid 0, reduction 1, prefix 2; odd: invalid 2,
// reduction 3, prefix 0, the reduction-to-prefix add wrapping 3 + 1 to 0 in 32 bits), the
// subgroup-size-1 ranking (each key its own subgroup, so the in-block rank is index order), the
// per-digit decoupled look-back over the partition words, the shared-memory reorder and the
// global store.  Buffer reads past a buffer's end return 0 and writes past it are dropped (wgpu's
// robust buffer access).  Two schedules of the workgroups are offered: 0 = one workgroup after
// another; 1 = every workgroup publishes its reduction first, then look-backs run from the last
// workgroup down, so each one accumulates reductions back to the first workgroup's prefix.  Both
// must give the same buffers.  The tests compare this with std::stable_sort (the oracle used for
// the CUDA sort) and with the CUDA sort itself.
#include <stdint.h>
#include <stdlib.h>

#include <vector>

namespace {

constexpr uint32_t kWg = 256;                  // histogram_wg_size = scatter_wg_size
constexpr uint32_t kRows = 15;                 // rs_histogram_block_rows = rs_scatter_block_rows
constexpr uint32_t kBlock = kWg * kRows;       // 3840 keyvals per workgroup
constexpr uint32_t kRadix = 256;               // rs_radix_size
constexpr uint32_t kLog2 = 8;                  // rs_radix_log2
constexpr uint32_t kKeyvalSize = 4;            // rs_keyval_size (32-bit keys)
constexpr uint32_t kMaskStatus = 0xC0000000u;  // rs_partition_mask_status
constexpr uint32_t kMaskCount = 0x3FFFFFFFu;   // rs_partition_mask_count

struct Buf {
    uint32_t *p;
    size_t len;
    uint32_t load(size_t i) const { return i < len ? p[i] : 0u; }
    void store(size_t i, uint32_t v) {
        if (i < len) p[i] = v;
    }
};

uint32_t digit_of(uint32_t v, uint32_t pass) { return (v >> (pass * kLog2)) & (kRadix - 1u); }

// prefix_reduce_smem (radix_sort.wgsl:173-200): in-place exclusive Blelloch scan of 256 words.
void prefix_reduce(uint32_t *smem) {
    uint32_t offset = 1;
    for (uint32_t d = kRadix >> 1; d > 0; d >>= 1) {
        for (uint32_t lid = 0; lid < d; ++lid) {
            const uint32_t ai = offset * (2 * lid + 1) - 1, bi = offset * (2 * lid + 2) - 1;
            smem[bi] += smem[ai];
        }
        offset <<= 1;
    }
    smem[kRadix - 1] = 0;
    for (uint32_t d = 1; d < kRadix; d <<= 1) {
        offset >>= 1;
        for (uint32_t lid = 0; lid < d; ++lid) {
            const uint32_t ai = offset * (2 * lid + 1) - 1, bi = offset * (2 * lid + 2) - 1;
            const uint32_t t = smem[ai];
            smem[ai] = smem[bi];
            smem[bi] += t;
        }
    }
}

// One workgroup of a scatter pass, split where the schedule may interleave workgroups: publish()
// loads, ranks and stores the reduction (or the first workgroup's prefix); finish() looks back,
// converts the reduction into a prefix, reorders and stores.
struct ScatterGroup {
    uint32_t kv[kWg][kRows], pv[kWg][kRows], kr[kWg][kRows];
    uint32_t smem[kRadix];      // the workgroup histogram, then its exclusive scan
    uint32_t lookback[kRadix];  // scatter_smem[0..256): exclusive global offset per digit
};

struct Pass {
    uint32_t pass, inv, red, pre;
    const Buf *in_k, *in_p;
    Buf *out_k, *out_p;
    uint32_t nwg;
    std::vector<uint32_t> *hist;  // histograms[4 x 256] then partitions[(blocks_ru - 1) x 256]
};

void publish(const Pass &P, uint32_t wid, ScatterGroup &g) {
    // fill_kv_even / fill_kv_odd with subgroup size 1: thread lid holds keys wid*3840 + lid*15 + i
    for (uint32_t lid = 0; lid < kWg; ++lid)
        for (uint32_t i = 0; i < kRows; ++i) {
            const size_t pos = (size_t)wid * kBlock + (size_t)lid * kRows + i;
            g.kv[lid][i] = P.in_k->load(pos);
            g.pv[lid][i] = P.in_p->load(pos);
        }
    // ranking with subgroups of one invocation: count = rank = 1 for every key
    for (uint32_t lid = 0; lid < kWg; ++lid)
        for (uint32_t i = 0; i < kRows; ++i) g.kr[lid][i] = (1u << 16) | 1u;
    // workgroup histogram, subgroup after subgroup (radix_sort.wgsl:323-343)
    for (uint32_t d = 0; d < kRadix; ++d) g.smem[d] = 0;
    for (uint32_t sg = 0; sg < kWg; ++sg)
        for (uint32_t j = 0; j < kRows; ++j) {
            const uint32_t digit = digit_of(g.kv[sg][j], P.pass);
            const uint32_t prev = g.smem[digit];
            const uint32_t rank = g.kr[sg][j] & 0xFFFFu, count = g.kr[sg][j] >> 16;
            g.kr[sg][j] = prev + rank;
            if (rank == count) g.smem[digit] = prev + count;
        }
    std::vector<uint32_t> &H = *P.hist;
    const size_t part0 = (size_t)kKeyvalSize * kRadix;
    for (uint32_t d = 0; d < kRadix; ++d) {
        const size_t at = part0 + (size_t)wid * kRadix + d;
        if (wid == 0) {
            const uint32_t exc = H[(size_t)P.pass * kRadix + d];
            g.lookback[d] = exc;
            if (at < H.size()) H[at] = (exc + g.smem[d]) | (P.pre << 30);
        } else if (wid < P.nwg - 1) {
            if (at < H.size()) H[at] = g.smem[d] | (P.red << 30);
        }
    }
}

bool finish(const Pass &P, uint32_t wid, ScatterGroup &g) {
    std::vector<uint32_t> &H = *P.hist;
    const size_t part0 = (size_t)kKeyvalSize * kRadix;
    if (wid > 0) {
        for (uint32_t d = 0; d < kRadix; ++d) {
            int64_t prev_wg = (int64_t)wid - 1;
            uint32_t exc = 0;
            for (;;) {
                if (prev_wg < 0) return false;  // no prefix below: the schedule broke the protocol
                const size_t at = part0 + (size_t)prev_wg * kRadix + d;
                const uint32_t prev = at < H.size() ? H[at] : 0u;
                // an unpublished predecessor: a serial schedule never meets one
                if ((prev & kMaskStatus) == (P.inv << 30)) return false;
                exc += prev & kMaskCount;
                if ((prev & kMaskStatus) != (P.pre << 30)) {
                    --prev_wg;
                    continue;
                }
                g.lookback[d] = exc;
                const size_t own = part0 + (size_t)wid * kRadix + d;
                if (wid < P.nwg - 1 && own < H.size()) H[own] += exc | (1u << 30);  // 32-bit wrap
                break;
            }
        }
    }
    prefix_reduce(g.smem);
    // rs_rank_to_local: 1-based local index in the upper half of kr
    for (uint32_t lid = 0; lid < kWg; ++lid)
        for (uint32_t i = 0; i < kRows; ++i) {
            const uint32_t digit = digit_of(g.kv[lid][i], P.pass);
            const uint32_t idx = g.smem[digit] + g.kr[lid][i];
            g.kr[lid][i] |= idx << 16;
        }
    // rs_reorder through shared memory: thread lid takes local slots lid, lid + 256, ...
    static thread_local uint32_t reorder_k[kBlock], reorder_p[kBlock], reorder_r[kBlock];
    for (uint32_t lid = 0; lid < kWg; ++lid)
        for (uint32_t j = 0; j < kRows; ++j) {
            const uint32_t slot = (g.kr[lid][j] >> 16) - 1u;
            if (slot >= kBlock) return false;
            reorder_k[slot] = g.kv[lid][j];
            reorder_p[slot] = g.pv[lid][j];
            reorder_r[slot] = g.kr[lid][j];
        }
    for (uint32_t lid = 0; lid < kWg; ++lid)
        for (uint32_t j = 0; j < kRows; ++j) {
            const uint32_t slot = lid + j * kWg;
            const uint32_t key = reorder_k[slot], pay = reorder_p[slot];
            const uint32_t rank = reorder_r[slot] & 0xFFFFu;
            // rs_local_to_global and rs_store
            const uint32_t global = rank + g.lookback[digit_of(key, P.pass)] - 1u;
            P.out_k->store(global, key);
            P.out_p->store(global, pay);
        }
    return true;
}

}  // namespace

extern "C" {

// keys: the GaussiansDepthBuffer contents (keys_len u32, at least keys_buffer_size(num_keys));
// payload: the IndirectIndicesBuffer (payload_len u32, N for the reference); num_keys: the
// sorter state's key count (N); dispatch_x: workgroups of the indirect dispatch (ceil(V / 3840)).
// Sorts in place like the reference; returns 0, or -1 if a look-back met an unpublished or
// missing predecessor (which would hang the reference).
int oracle_wgpu_radix_sort(uint32_t *keys, uint32_t keys_len, uint32_t *payload, uint32_t payload_len,
                           uint32_t num_keys, uint32_t dispatch_x, int schedule) {
    const uint32_t blocks_ru = (num_keys + kBlock - 1) / kBlock;                 // scatter_blocks_ru
    const uint32_t padded = blocks_ru * kBlock;                                  // keys_buffer_size
    std::vector<uint32_t> keys_b((size_t)padded * kKeyvalSize, 0u);             // keys_aux
    std::vector<uint32_t> payload_b(num_keys, 0u);                              // payload_aux
    std::vector<uint32_t> hist((size_t)(kKeyvalSize + blocks_ru) * kRadix, 0u);  // internal buffer
    Buf ka{keys, keys_len}, kb{keys_b.data(), keys_b.size()}, pa{payload, payload_len}, pb{payload_b.data(), payload_b.size()};
    if (dispatch_x == 0) return 0;  // no workgroup runs
    // zero_histograms (radix_sort.wgsl:78-112)
    {
        const size_t n = (size_t)(kKeyvalSize + blocks_ru - 1) * kRadix;
        for (size_t i = 0; i < n && i < hist.size(); ++i) hist[i] = 0u;
        for (uint32_t i = num_keys; i < padded; ++i) ka.store(i, 0xFFFFFFFFu);
    }
    // calculate_histogram (radix_sort.wgsl:117-168): fill_kv reads keys wid*3840 + lid + i*256
    for (uint32_t wid = 0; wid < dispatch_x; ++wid)
        for (uint32_t pass = 0; pass < kKeyvalSize; ++pass)
            for (uint32_t lid = 0; lid < kWg; ++lid)
                for (uint32_t i = 0; i < kRows; ++i) {
                    const uint32_t v = ka.load((size_t)wid * kBlock + lid + (size_t)i * kWg);
                    if ((size_t)pass * kRadix + digit_of(v, pass) < hist.size()) ++hist[(size_t)pass * kRadix + digit_of(v, pass)];
                }
    // prefix_histogram (radix_sort.wgsl:202-220)
    for (uint32_t pass = 0; pass < kKeyvalSize; ++pass) prefix_reduce(hist.data() + (size_t)pass * kRadix);
    // scatter_even / scatter_odd / scatter_even / scatter_odd (radix_sort.wgsl:482-529):
    // infos.even_pass starts 0 and odd_pass 1, each kernel's first invocation flips the other one
    uint32_t even_pass = 0, odd_pass = 1;
    std::vector<ScatterGroup> groups(schedule == 1 ? dispatch_x : 1);
    for (int k = 0; k < 4; ++k) {
        const bool even = (k % 2) == 0;
        Pass P;
        if (even) {
            odd_pass = (odd_pass + 1u) % 2u;
            P.pass = even_pass * 2u;
            P.inv = 0u, P.red = 1u, P.pre = 2u;
            P.in_k = &ka, P.in_p = &pa, P.out_k = &kb, P.out_p = &pb;
        } else {
            even_pass = (even_pass + 1u) % 2u;
            P.pass = odd_pass * 2u + 1u;
            P.inv = 2u, P.red = 3u, P.pre = 0u;
            P.in_k = &kb, P.in_p = &pb, P.out_k = &ka, P.out_p = &pa;
        }
        P.nwg = dispatch_x;
        P.hist = &hist;
        if (schedule == 1) {
            for (uint32_t wid = 0; wid < dispatch_x; ++wid) publish(P, wid, groups[wid]);
            if (!finish(P, 0, groups[0])) return -1;
            for (uint32_t wid = dispatch_x; wid-- > 1;)
                if (!finish(P, wid, groups[wid])) return -1;
        } else {
            for (uint32_t wid = 0; wid < dispatch_x; ++wid) {
                publish(P, wid, groups[0]);
                if (!finish(P, wid, groups[0])) return -1;
            }
        }
    }
    return 0;
}

}  // extern "C"
