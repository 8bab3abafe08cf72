// zf_syntax.cpp -- the tile symbol coder and the filter stage's tile syntax
// written through it: per-superblock loop-restoration units and per-filter-
// block cdef_idx literals, as bytes.
//
// The coder is AV1's multi-symbol arithmetic coder, the encoder side of the
// specification's symbol decoding process (AV1 spec 8.2.2-8.2.6), which the
// reference wraps as AomWriter over OdEcEnc (svtav1-entropy/src/writer.rs:
// 18-80, range_coder.rs:24-300). Interval arithmetic and CDF adaptation are
// normative (the decoder must track them exactly); the final flush follows
// the reference's rule (range_coder.rs:207-258) so the bytes are the same:
// the code value is the low end rounded up to a multiple of 2^14 window
// units with the 2^14 bit set, written through the stream bit that bit
// lands on, the last byte zero-padded.
//
// Representation. `low` holds the code value's bits that are not yet in
// `out`: its bit i is stream bit (14 + pos - i), where pos counts the
// renormalisation shifts so far, so the 16-bit coding window is low's bits
// 15..0 and stream bit 0 starts at window bit 14 (the range starts at
// 2^15). A byte leaves `low` as soon as all its bits are above the window
// (pos >= 8 * bytes + 9); an addition that carries past the bits still held
// ripples into the bytes already written.
#include <cstdint>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/zf_filter.h"

struct zf_ec {
    std::vector<uint8_t> out;
    uint64_t low = 0;
    uint32_t rng = 0x8000;
    int64_t pos = 0;
};

namespace {

constexpr int kProbShift = 6;  // EC_PROB_SHIFT (spec 8.2.6)
constexpr uint32_t kMinProb = 4;  // EC_MIN_PROB

int bit_length(uint32_t v) { return v ? 32 - __builtin_clz(v) : 0; }

// The carry bit sits just above the highest stream bit still held in low.
void settle_carry(zf_ec &e) {
    const int64_t top = 15 + e.pos - 8 * (int64_t)e.out.size();
    if (top >= 64 || !((e.low >> top) & 1)) return;
    e.low &= ~(1ull << top);
    for (size_t i = e.out.size(); i-- > 0;)
        if (++e.out[i] != 0) break;  // a carry out of byte 0 cannot occur: the code value stays below 1
}

void renormalise(zf_ec &e) {
    const int d = 16 - bit_length(e.rng);
    e.low <<= d;
    e.rng <<= d;
    e.pos += d;
    while (e.pos >= 8 * (int64_t)e.out.size() + 9) {
        const int sh = (int)(7 + e.pos - 8 * (int64_t)e.out.size());
        e.out.push_back((uint8_t)(e.low >> sh));
        e.low &= (1ull << sh) - 1;
    }
}

// Symbol s of nsyms under the inverse CDF icdf (C layout: icdf[i] =
// 32768 - P(x <= i) in Q15, icdf[nsyms - 1] = 0). The decoder's threshold
// for "x > i" is ((rng >> 8) * (icdf[i] >> 6) >> 1) + 4 * (nsyms - 1 - i);
// symbol s owns [threshold(s), threshold(s - 1)) counted from the top.
void code_symbol(zf_ec &e, int s, const uint16_t *icdf, int nsyms) {
    auto thr = [&](int i) -> uint32_t {
        return (((e.rng >> 8) * (uint32_t)(icdf[i] >> kProbShift)) >> (7 - kProbShift)) +
               kMinProb * (uint32_t)(nsyms - 1 - i);
    };
    const uint32_t hi = s > 0 ? thr(s - 1) : e.rng;
    const uint32_t lo = thr(s);
    e.low += e.rng - hi;
    e.rng = hi - lo;
    settle_carry(e);
    renormalise(e);
}

// CDF adaptation after coding s (spec 8.2.6, in inverse-CDF form): the
// counter at icdf[nsyms] sets the rate 4 + (count > 15) + (count > 31),
// one more above three symbols.
void adapt(uint16_t *icdf, int s, int nsyms) {
    const int count = icdf[nsyms];
    const int rate = 4 + (count > 15) + (count > 31) + (nsyms > 3);
    for (int i = 0; i < nsyms - 1; ++i) {
        if (i < s)
            icdf[i] = (uint16_t)(icdf[i] + ((32768 - icdf[i]) >> rate));
        else
            icdf[i] = (uint16_t)(icdf[i] - (icdf[i] >> rate));
    }
    if (count < 32) icdf[nsyms] = (uint16_t)(count + 1);
}

void code_bool(zf_ec &e, int bit, uint32_t f) {
    const uint16_t icdf[2] = {(uint16_t)f, 0};
    code_symbol(e, bit ? 1 : 0, icdf, 2);
}

void code_literal(zf_ec &e, uint32_t v, int nbits) {
    for (int b = nbits - 1; b >= 0; --b) code_bool(e, (v >> b) & 1, 16384);
}

}  // namespace

zf_ec *zf_ec_create(void) { return new (std::nothrow) zf_ec(); }

void zf_ec_destroy(zf_ec *ec) { delete ec; }

void zf_ec_reset(zf_ec *ec) {
    if (ec) *ec = zf_ec();
}

int32_t zf_ec_bool(zf_ec *ec, int32_t bit, uint32_t f) {
    if (!ec || f == 0 || f >= 32768) return ZF_ERR_ARG;
    code_bool(*ec, bit, f);
    return ZF_OK;
}

int32_t zf_ec_literal(zf_ec *ec, uint32_t value, int32_t nbits) {
    if (!ec || nbits < 0 || nbits > 32) return ZF_ERR_ARG;
    code_literal(*ec, value, nbits);
    return ZF_OK;
}

int32_t zf_ec_symbol(zf_ec *ec, int32_t s, uint16_t *icdf, int32_t nsyms, int32_t adapt_cdf) {
    if (!ec || !icdf || nsyms < 2 || nsyms > 16 || s < 0 || s >= nsyms || icdf[nsyms - 1] != 0) return ZF_ERR_ARG;
    for (int i = 1; i < nsyms; ++i)
        if (icdf[i] > icdf[i - 1] || icdf[i - 1] > 32768) return ZF_ERR_ARG;
    code_symbol(*ec, s, icdf, nsyms);
    if (adapt_cdf) adapt(icdf, s, nsyms);
    return ZF_OK;
}

int32_t zf_ec_tell(const zf_ec *ec) { return ec ? (int32_t)(ec->pos + 1) : ZF_ERR_ARG; }

int32_t zf_ec_done(zf_ec *ec, uint8_t *out, int32_t cap) {
    if (!ec || (!out && cap > 0) || cap < 0) return ZF_ERR_ARG;
    const int64_t total = (ec->pos + 1 + 7) / 8;
    if (total > cap) return ZF_ERR_ARG;
    zf_ec e = *ec;  // the coder itself stays open: more symbols may follow
    e.low = ((e.low + 0x3FFF) & ~0x3FFFull) | 0x4000;
    settle_carry(e);
    for (int64_t j = (int64_t)e.out.size(); j < total; ++j) {
        const int64_t sh = 7 + e.pos - 8 * j;
        e.out.push_back((uint8_t)(sh >= 0 ? e.low >> sh : e.low << -sh));
    }
    std::memcpy(out, e.out.data(), (size_t)total);
    return (int32_t)total;
}

void zf_wiener_restore_cdf_init(uint16_t cdf[3]) {
    cdf[0] = 32768 - 11570;  // Default_Use_Wiener_Cdf (AV1 spec; svtav1-entropy/src/context.rs:544)
    cdf[1] = 0;
    cdf[2] = 0;
}

int32_t zf_ec_lr_syms(zf_ec *ec, const zf_lr_sym *syms, int32_t n, uint16_t wiener_cdf[3]) {
    if (!ec || (!syms && n > 0) || n < 0 || !wiener_cdf || wiener_cdf[1] != 0) return ZF_ERR_ARG;
    for (int i = 0; i < n; ++i)
        if (!((syms[i].kind == ZF_SYM_WIENER_RESTORE && syms[i].value <= 1) ||
              (syms[i].kind == ZF_SYM_BITS && syms[i].nbits >= 1 && syms[i].nbits <= 16)))
            return ZF_ERR_ARG;
    for (int i = 0; i < n; ++i) {
        if (syms[i].kind == ZF_SYM_WIENER_RESTORE) {
            code_symbol(*ec, (int)syms[i].value, wiener_cdf, 2);
            adapt(wiener_cdf, (int)syms[i].value, 2);
        } else {
            code_literal(*ec, syms[i].value, syms[i].nbits);
        }
    }
    return ZF_OK;
}

int32_t zf_ec_lr_sb(zf_ec *ec, const zf_decisions *d, int32_t mi_row, int32_t mi_col, int32_t sb_mi, int32_t frame_w,
                    int32_t frame_h, int32_t monochrome, int32_t sr_denom, zf_wiener_refs *refs, uint16_t wiener_cdf[3]) {
    if (!ec || !wiener_cdf || !refs) return ZF_ERR_ARG;
    // a 128x128 superblock holds the corners of at most 5 x 5 units of a
    // plane (32-sample units), each a flag and six taps of at most five
    // elements (a few more-bits, then the value)
    std::vector<zf_lr_sym> syms(3 * 25 * 32);
    zf_wiener_refs r = *refs;
    const int n = zf_lr_sb_syntax(d, mi_row, mi_col, sb_mi, frame_w, frame_h, monochrome, sr_denom, &r, syms.data(),
                                  (int32_t)syms.size());
    if (n < 0) return n;
    const int rc = zf_ec_lr_syms(ec, syms.data(), n, wiener_cdf);
    if (rc == ZF_OK) *refs = r;
    return rc == ZF_OK ? n : rc;
}

int32_t zf_cdef_sb_begin(const zf_decisions *d, int32_t sb_row, int32_t sb_col, int32_t sb_size, zf_cdef_sb *st) {
    if (!d || !st || sb_row < 0 || sb_col < 0 || (sb_size != 64 && sb_size != 128)) return ZF_ERR_ARG;
    if (d->cdef_bits > 3 || (d->cdef_bits > 0 && !d->cdef_fb_idx)) return ZF_ERR_ARG;
    std::memset(st, 0, sizeof(*st));
    st->bits = d->cdef_bits;
    st->sb128 = sb_size == 128;
    const int per = sb_size / 64;
    for (int q = 0; q < 4; ++q) {
        const int fbc = sb_col * per + (q & 1), fbr = sb_row * per + (q >> 1);
        // quadrants outside the frame code nothing; 0 keeps the slot defined
        if (d->cdef_bits > 0 && fbc < d->nhfb && fbr < d->nvfb) st->strengths[q] = d->cdef_fb_idx[fbr * d->nhfb + fbc];
    }
    return ZF_OK;
}

int32_t zf_ec_cdef_block(zf_ec *ec, zf_cdef_sb *st, int32_t block_x, int32_t block_y, int32_t skip) {
    if (!ec || !st || block_x < 0 || block_y < 0) return ZF_ERR_ARG;
    if (skip || st->bits == 0) return 0;
    const int q = st->sb128 ? ((block_x >> 6) & 1) + 2 * ((block_y >> 6) & 1) : 0;
    if (st->transmitted[q]) return 0;
    st->transmitted[q] = 1;
    code_literal(*ec, st->strengths[q], st->bits);
    return st->bits;
}
