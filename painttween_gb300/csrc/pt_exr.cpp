// pt_exr.cpp -- the Huffman stage of OpenEXR's PIZ codec, decoding side
// (pt_piz_huffman_decode), for reading the reference's PIZ-compressed
// temporary images.  Written from the published layout of a PIZ Huffman
// block:
//   u32 im, iM      first and last symbol of the code-length table; iM is the
//                   run symbol (one above the largest word)
//   u32 table bytes, u32 bit count, u32 0
//   table           6-bit code lengths of im..iM, most significant bit first;
//                   59..62 stand for runs of 2..5 zero lengths, 63 followed
//                   by 8 bits n for n + 6 zero lengths
//   bits            the codes, most significant bit first
// Codes are canonical, assigned from the longest length down: the lowest
// code of length l follows from the counts of all longer lengths, and
// within a length the codes rise with the symbol.  The run symbol is
// followed by 8 bits r: the word before it is repeated r more times.
#include <cstdint>
#include <cstring>
#include <vector>

#include "painttween.h"

namespace {

constexpr int kMaxLen = 58;
constexpr int kFastBits = 14;  // codes up to this long are decoded by one table lookup

struct BitReader {
    const uint8_t* p;
    const uint8_t* end;
    uint64_t c = 0;  // pending bits, the oldest highest
    int n = 0;       // pending bit count
    bool over = false;
    // makes at least k (<= 56) bits pending; past the end they read as 0
    void need(int k) {
        while (n < k) {
            uint8_t b = 0;
            if (p < end)
                b = *p++;
            else
                over = true;
            c = (c << 8) | b;
            n += 8;
        }
    }
    uint64_t get(int k) {
        need(k);
        n -= k;
        const uint64_t v = (c >> n) & ((k == 64) ? ~0ull : ((1ull << k) - 1));
        c &= (n ? ((1ull << n) - 1) : 0);
        return v;
    }
};

uint32_t rd32(const uint8_t* p) { return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24); }

}  // namespace

pt_status pt_piz_huffman_decode(const uint8_t* block, size_t block_bytes, uint16_t* out, size_t n_words) {
    if (block_bytes == 0) return n_words == 0 ? PT_OK : PT_ERR_INVALID;
    if (!block || (n_words && !out) || block_bytes < 20) return PT_ERR_INVALID;
    const uint32_t im = rd32(block), iM = rd32(block + 4), nbits = rd32(block + 12);
    if (im > 65536 || iM > 65536 || im > iM) return PT_ERR_INVALID;

    // code lengths
    std::vector<uint8_t> len(iM + 1, 0);
    BitReader tr{block + 20, block + block_bytes};
    for (uint32_t i = im; i <= iM;) {
        const int l = (int)tr.get(6);
        if (tr.over) return PT_ERR_INVALID;
        if (l >= 59) {
            const uint32_t run = (l == 63) ? (uint32_t)tr.get(8) + 6 : (uint32_t)(l - 59 + 2);
            if (tr.over || i + run > iM + 1) return PT_ERR_INVALID;
            i += run;
        } else {
            len[i++] = (uint8_t)l;
        }
    }
    const uint8_t* data = tr.p;  // the table ends at a byte boundary
    if ((uint64_t)nbits > (uint64_t)(block + block_bytes - data) * 8) return PT_ERR_INVALID;

    // canonical codes
    uint64_t count[kMaxLen + 1] = {0}, first[kMaxLen + 1] = {0};
    for (uint32_t s = im; s <= iM; s++) count[len[s]]++;
    count[0] = 0;
    uint64_t c = 0;
    for (int l = kMaxLen; l > 0; l--) {
        first[l] = c;
        c = (c + count[l]) >> 1;
    }
    // per length: its symbols in code order (rising symbol)
    std::vector<uint32_t> offset(kMaxLen + 2, 0);
    for (int l = 1; l <= kMaxLen; l++) offset[l + 1] = offset[l] + (uint32_t)count[l];
    std::vector<uint32_t> sorted(offset[kMaxLen + 1]);
    {
        std::vector<uint32_t> fill(offset.begin(), offset.end());
        for (uint32_t s = im; s <= iM; s++)
            if (len[s]) sorted[fill[len[s]]++] = s;
    }
    int maxlen = 0;
    for (int l = 1; l <= kMaxLen; l++) {
        if (!count[l]) continue;
        maxlen = l;
        if (first[l] + count[l] > (1ull << l)) return PT_ERR_INVALID;  // not a prefix code
    }
    // a chunk holds far fewer than 2^32 words, which bounds its Huffman codes
    // well below 56 bits (the reader's window); longer ones are rejected
    if (!maxlen || maxlen > 56) return PT_ERR_INVALID;
    // one-lookup table of the codes up to kFastBits long: (symbol << 8) | length
    std::vector<uint32_t> fast(1u << kFastBits, 0);
    for (int l = 1; l <= kFastBits && l <= maxlen; l++) {
        for (uint64_t k = 0; k < count[l]; k++) {
            const uint32_t sym = sorted[offset[l] + k];
            const uint64_t lo = (first[l] + k) << (kFastBits - l);
            for (uint64_t j = 0; j < (1ull << (kFastBits - l)); j++) fast[lo + j] = (sym << 8) | (uint32_t)l;
        }
    }

    BitReader br{data, block + block_bytes};
    uint64_t used = 0;
    size_t o = 0;
    while (used < nbits) {
        br.need(maxlen < kFastBits ? kFastBits : maxlen);
        // the next kFastBits bits
        const uint32_t top = (uint32_t)((br.c >> (br.n - kFastBits)) & ((1u << kFastBits) - 1));
        uint32_t sym = 0;
        int l = 0;
        if (fast[top]) {
            sym = fast[top] >> 8;
            l = (int)(fast[top] & 0xFF);
        } else {  // a longer code: canonical search by length
            for (int k = kFastBits + 1; k <= maxlen; k++) {
                const uint64_t v = (br.c >> (br.n - k)) & ((1ull << k) - 1);
                if (count[k] && v >= first[k] && v - first[k] < count[k]) {
                    sym = sorted[offset[k] + (uint32_t)(v - first[k])];
                    l = k;
                    break;
                }
            }
            if (!l) return PT_ERR_INVALID;
        }
        br.get(l);
        used += (uint64_t)l;
        if (sym == iM) {  // run: the previous word r more times
            const uint32_t r = (uint32_t)br.get(8);
            used += 8;
            if (o == 0 || o + r > n_words) return PT_ERR_INVALID;
            const uint16_t w = out[o - 1];
            for (uint32_t k = 0; k < r; k++) out[o++] = w;
        } else {
            if (o >= n_words || sym > 65535) return PT_ERR_INVALID;
            out[o++] = (uint16_t)sym;
        }
    }
    if (used != nbits || o != n_words) return PT_ERR_INVALID;
    return PT_OK;
}
