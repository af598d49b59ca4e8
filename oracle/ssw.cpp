// Oracle (test infrastructure only): striped Smith-Waterman, CIGAR handling and
// the aligner front end.
//
// ssw_align restates the vendored SSW library (ext/ssw/ssw.c, MIT) lane for lane:
// the query profile is laid out in Farrar's striped order (16 x u8 lanes in
// "byte" mode, 8 x i16 lanes in "word" mode), the lazy-F pass does not update E,
// and byte mode is abandoned for word mode once max + bias >= 255.  Emulating the
// stripes is required for bit-exactness: which cells receive their vertical-gap
// value in the main pass (and so also feed E) depends on segLen.
// Also restates src/ssw.rs, src/cigar.rs and src/aligner.rs.
#include "oracle.hpp"

#include <algorithm>
#include <cstdlib>
#include <stdexcept>

namespace oracle {

// ------------------------------------------------------------------ CIGAR
// src/cigar.rs:100-187
void Cigar::push(uint8_t op, size_t len) {
    if (len == 0) return;
    if (!ops.empty() && (ops.back() & 15) == op) ops.back() += (uint32_t)(len << 4);
    else ops.push_back((uint32_t)(len << 4) | op);
}

Cigar Cigar::reversed() const {
    Cigar c;
    c.ops.assign(ops.rbegin(), ops.rend());
    return c;
}

Cigar Cigar::with_m() const {
    Cigar c;
    for (uint32_t v : ops) {
        uint8_t op = v & 15;
        if (op == OP_EQ || op == OP_X) op = OP_M;
        c.push(op, v >> 4);
    }
    return c;
}

Cigar Cigar::with_eqx(const std::string& q, const std::string& r) const {
    Cigar c;
    size_t qi = 0, ri = 0;
    for (uint32_t v : ops) {
        uint8_t op = v & 15;
        size_t len = v >> 4;
        switch (op) {
            case OP_M:
                for (size_t t = 0; t < len; t++) {
                    c.push(q.at(qi) == r.at(ri) ? OP_EQ : OP_X, 1);
                    qi++;
                    ri++;
                }
                break;
            case OP_I: case OP_S: c.push(op, len); qi += len; break;
            case OP_D: case OP_N: c.push(op, len); ri += len; break;
            case OP_H: case OP_P: c.push(op, len); break;
            default: c.push(op, len); qi += len; ri += len; break;
        }
    }
    return c;
}

size_t Cigar::edit_distance() const {
    size_t d = 0;
    for (uint32_t v : ops) {
        uint8_t op = v & 15;
        if (op == OP_X || op == OP_I || op == OP_D) d += v >> 4;
    }
    return d;
}

std::string Cigar::str() const {
    static const char* ch = "MIDNSHP=X";
    std::string s;
    for (uint32_t v : ops) {
        s += std::to_string(v >> 4);
        s += ch[v & 15];
    }
    return s;
}

// ------------------------------------------------------------------ SSW
static inline uint8_t addus8(uint8_t a, uint8_t b) { unsigned s = (unsigned)a + b; return s > 255 ? 255 : (uint8_t)s; }
static inline uint8_t subus8(uint8_t a, uint8_t b) { return a > b ? (uint8_t)(a - b) : 0; }
static inline int16_t adds16(int16_t a, int16_t b) {
    int s = (int)a + (int)b;
    return (int16_t)std::clamp(s, -32768, 32767);
}
static inline int16_t subus16(int16_t a, int16_t b) {
    uint16_t x = (uint16_t)a, y = (uint16_t)b;
    return x > y ? (int16_t)(uint16_t)(x - y) : 0;
}

struct EndPos {
    uint16_t score;
    int32_t ref, read;
};

// ext/ssw/ssw.c:138-161 (qP_byte): profile[nt][seg][lane]
static std::vector<uint8_t> profile_byte(const int8_t* read, const int8_t* mat, int32_t len, int32_t n, uint8_t bias) {
    int32_t seg = (len + 15) / 16;
    std::vector<uint8_t> p((size_t)n * seg * 16);
    size_t t = 0;
    for (int32_t nt = 0; nt < n; nt++)
        for (int32_t i = 0; i < seg; i++)
            for (int32_t lane = 0, j = i; lane < 16; lane++, j += seg)
                p[t++] = (uint8_t)(j >= len ? bias : (int8_t)(mat[nt * n + read[j]] + bias));
    return p;
}

// ext/ssw/ssw.c:393-413 (qP_word)
static std::vector<int16_t> profile_word(const int8_t* read, const int8_t* mat, int32_t len, int32_t n) {
    int32_t seg = (len + 7) / 8;
    std::vector<int16_t> p((size_t)n * seg * 8);
    size_t t = 0;
    for (int32_t nt = 0; nt < n; nt++)
        for (int32_t i = 0; i < seg; i++)
            for (int32_t lane = 0, j = i; lane < 8; lane++, j += seg)
                p[t++] = (int16_t)(j >= len ? 0 : mat[nt * n + read[j]]);
    return p;
}

// ext/ssw/ssw.c:169-390 (sw_sse2_byte), scalar lanes
static EndPos sw_byte(const int8_t* ref, bool reverse, int32_t ref_len, int32_t read_len, uint8_t gap_o,
                      uint8_t gap_e, const std::vector<uint8_t>& prof, uint8_t terminate, uint8_t bias) {
    const int32_t seg = (read_len + 15) / 16;
    uint8_t max = 0;
    int32_t end_read = read_len - 1, end_ref = -1;
    std::vector<uint8_t> b1(seg * 16, 0), b2(seg * 16, 0), E(seg * 16, 0), Hmax(seg * 16, 0);
    uint8_t* Hs = b1.data();
    uint8_t* Hl = b2.data();
    uint8_t vMaxScore[16] = {0}, vMaxMark[16] = {0};
    int32_t begin = 0, end = ref_len, step = 1;
    if (reverse) { begin = ref_len - 1; end = -1; step = -1; }
    for (int32_t i = begin; i != end; i += step) {
        uint8_t vF[16] = {0}, vMaxCol[16] = {0}, vH[16];
        vH[0] = 0;
        for (int l = 1; l < 16; l++) vH[l] = Hs[(seg - 1) * 16 + l - 1];
        std::swap(Hs, Hl);
        const uint8_t* P = prof.data() + (size_t)ref[i] * seg * 16;
        for (int32_t j = 0; j < seg; j++) {
            for (int l = 0; l < 16; l++) {
                uint8_t h = subus8(addus8(vH[l], P[j * 16 + l]), bias);
                uint8_t e = E[j * 16 + l];
                h = std::max(h, e);
                h = std::max(h, vF[l]);
                vMaxCol[l] = std::max(vMaxCol[l], h);
                Hs[j * 16 + l] = h;
                h = subus8(h, gap_o);
                e = std::max(subus8(e, gap_e), h);
                E[j * 16 + l] = e;
                vF[l] = std::max(subus8(vF[l], gap_e), h);
                vH[l] = Hl[j * 16 + l];
            }
        }
        bool done = false;
        for (int k = 0; k < 16 && !done; k++) {
            for (int l = 15; l > 0; l--) vF[l] = vF[l - 1];
            vF[0] = 0;
            for (int32_t j = 0; j < seg; j++) {
                bool settled = true;
                for (int l = 0; l < 16; l++) {
                    uint8_t h = std::max(Hs[j * 16 + l], vF[l]);
                    vMaxCol[l] = std::max(vMaxCol[l], h);
                    Hs[j * 16 + l] = h;
                    h = subus8(h, gap_o);
                    vF[l] = subus8(vF[l], gap_e);
                    if (subus8(vF[l], h) != 0) settled = false;
                }
                if (settled) { done = true; break; }
            }
        }
        bool changed = false;
        for (int l = 0; l < 16; l++) {
            vMaxScore[l] = std::max(vMaxScore[l], vMaxCol[l]);
            if (vMaxScore[l] != vMaxMark[l]) changed = true;
        }
        if (changed) {
            uint8_t temp = 0;
            for (int l = 0; l < 16; l++) { vMaxMark[l] = vMaxScore[l]; temp = std::max(temp, vMaxScore[l]); }
            if (temp > max) {
                max = temp;
                if ((int)max + bias >= 255) break;
                end_ref = i;
                std::copy(Hs, Hs + seg * 16, Hmax.begin());
            }
        }
        uint8_t colmax = 0;
        for (int l = 0; l < 16; l++) colmax = std::max(colmax, vMaxCol[l]);
        if (colmax == terminate) break;
    }
    for (int32_t t = 0; t < seg * 16; t++) {
        if (Hmax[t] == max) {
            int32_t pos = t / 16 + (t % 16) * seg;
            if (pos < end_read) end_read = pos;
        }
    }
    EndPos r;
    r.score = ((int)max + bias >= 255) ? 255 : max;
    r.ref = end_ref;
    r.read = end_read;
    return r;
}

// ext/ssw/ssw.c:415-596 (sw_sse2_word), scalar lanes
static EndPos sw_word(const int8_t* ref, bool reverse, int32_t ref_len, int32_t read_len, uint8_t gap_o,
                      uint8_t gap_e, const std::vector<int16_t>& prof, uint16_t terminate) {
    const int32_t seg = (read_len + 7) / 8;
    uint16_t max = 0;
    int32_t end_read = read_len - 1, end_ref = 0;
    std::vector<int16_t> b1(seg * 8, 0), b2(seg * 8, 0), E(seg * 8, 0), Hmax(seg * 8, 0);
    int16_t* Hs = b1.data();
    int16_t* Hl = b2.data();
    int16_t vMaxScore[8] = {0}, vMaxMark[8] = {0};
    const int16_t go = gap_o, ge = gap_e;
    int32_t begin = 0, end = ref_len, step = 1;
    if (reverse) { begin = ref_len - 1; end = -1; step = -1; }
    for (int32_t i = begin; i != end; i += step) {
        int16_t vF[8] = {0}, vMaxCol[8] = {0}, vH[8];
        vH[0] = 0;
        for (int l = 1; l < 8; l++) vH[l] = Hs[(seg - 1) * 8 + l - 1];
        std::swap(Hs, Hl);
        const int16_t* P = prof.data() + (size_t)ref[i] * seg * 8;
        for (int32_t j = 0; j < seg; j++) {
            for (int l = 0; l < 8; l++) {
                int16_t h = adds16(vH[l], P[j * 8 + l]);
                int16_t e = E[j * 8 + l];
                h = std::max(h, e);
                h = std::max(h, vF[l]);
                vMaxCol[l] = std::max(vMaxCol[l], h);
                Hs[j * 8 + l] = h;
                h = subus16(h, go);
                e = std::max(subus16(e, ge), h);
                E[j * 8 + l] = e;
                vF[l] = std::max(subus16(vF[l], ge), h);
                vH[l] = Hl[j * 8 + l];
            }
        }
        bool done = false;
        for (int k = 0; k < 8 && !done; k++) {
            for (int l = 7; l > 0; l--) vF[l] = vF[l - 1];
            vF[0] = 0;
            for (int32_t j = 0; j < seg; j++) {
                bool any_gt = false;
                for (int l = 0; l < 8; l++) {
                    int16_t h = std::max(Hs[j * 8 + l], vF[l]);
                    vMaxCol[l] = std::max(vMaxCol[l], h);
                    Hs[j * 8 + l] = h;
                    h = subus16(h, go);
                    vF[l] = subus16(vF[l], ge);
                    if (vF[l] > h) any_gt = true;
                }
                if (!any_gt) { done = true; break; }
            }
        }
        bool changed = false;
        for (int l = 0; l < 8; l++) {
            vMaxScore[l] = std::max(vMaxScore[l], vMaxCol[l]);
            if (vMaxScore[l] != vMaxMark[l]) changed = true;
        }
        if (changed) {
            int16_t temp = vMaxScore[0];
            for (int l = 0; l < 8; l++) { vMaxMark[l] = vMaxScore[l]; temp = std::max(temp, vMaxScore[l]); }
            if ((uint16_t)temp > max) {
                max = (uint16_t)temp;
                end_ref = i;
                std::copy(Hs, Hs + seg * 8, Hmax.begin());
            }
        }
        int16_t colmax = vMaxCol[0];
        for (int l = 0; l < 8; l++) colmax = std::max(colmax, vMaxCol[l]);
        if ((uint16_t)colmax == terminate) break;
    }
    for (int32_t t = 0; t < seg * 8; t++) {
        if ((uint16_t)Hmax[t] == max) {
            int32_t pos = t / 8 + (t % 8) * seg;
            if (pos < end_read) end_read = pos;
        }
    }
    return EndPos{max, end_ref, end_read};
}

// ext/ssw/ssw.c:598-769 (banded_sw): banded global DP + traceback with band
// doubling.  Returns false where the reference takes its error exit or would read
// a direction cell that the last band pass did not write.
static bool banded_sw(const int8_t* ref, const int8_t* read, int32_t ref_len, int32_t read_len, int32_t score,
                      int32_t gap_o, int32_t gap_e, int32_t band_width, const int8_t* mat, int32_t n,
                      std::vector<uint32_t>& out) {
    int32_t max = 0, width = 0, width_d = 0;
    const int32_t len = std::max(ref_len, read_len);
    std::vector<int32_t> h_b, e_b, h_c;
    std::vector<int8_t> dir;
    do {
        width = band_width * 2 + 3;
        width_d = band_width * 2 + 1;
        h_b.assign(width + 1, 0);
        e_b.assign(width + 1, 0);
        h_c.assign(width + 1, 0);
        dir.assign((size_t)width_d * read_len * 3, 0);
        for (int32_t i = 0; i < read_len; i++) {
            int32_t beg = std::max(0, i - band_width), end = std::min(ref_len - 1, i + band_width);
            int32_t edge = std::min(end + 1, width - 1);
            int32_t f = 0, u = 0;
            h_b[0] = e_b[0] = h_b[edge] = e_b[edge] = h_c[0] = 0;
            int8_t* line = dir.data() + (size_t)width_d * i * 3;
            const int32_t x = std::max(i - band_width, 0), xe = std::max(i - 1 - band_width, 0);
            for (int32_t j = beg; j <= end; j++) {
                u = j - x + 1;
                int32_t e = j - xe + 1, b = j - x, d = j - xe;
                int32_t de = (j - x) * 3, df = de + 1, dh = de + 2;
                int32_t t1 = i == 0 ? -gap_o : h_b[e] - gap_o;
                int32_t t2 = i == 0 ? -gap_e : e_b[e] - gap_e;
                e_b[u] = t1 > t2 ? t1 : t2;
                line[de] = t1 > t2 ? 3 : 2;
                t1 = h_c[b] - gap_o;
                t2 = f - gap_e;
                f = t1 > t2 ? t1 : t2;
                line[df] = t1 > t2 ? 5 : 4;
                int32_t e1 = e_b[u] > 0 ? e_b[u] : 0, f1 = f > 0 ? f : 0;
                t1 = e1 > f1 ? e1 : f1;
                t2 = h_b[d] + mat[ref[j] * n + read[i]];
                h_c[u] = t1 > t2 ? t1 : t2;
                if (h_c[u] > max) max = h_c[u];
                if (t1 <= t2) line[dh] = 1;
                else line[dh] = e1 > f1 ? line[de] : line[df];
            }
            for (int32_t j = 1; j <= u; j++) h_b[j] = h_c[j];
        }
        band_width *= 2;
    } while (max < score && band_width <= len);
    band_width /= 2;

    int32_t i = read_len - 1, j = ref_len - 1, e = 0;
    int64_t line = (int64_t)width_d * i * 3;
    char op = 'M', prev = 'M';
    int32_t which = 2;
    std::vector<uint32_t> c;
    auto enc = [](int32_t l, char o) { return (uint32_t)l << 4 | (o == 'M' ? 0u : o == 'I' ? 1u : 2u); };
    while (i >= 0 && j > 0) {
        int32_t x = std::max(i - band_width, 0);
        int64_t at = line + (int64_t)(j - x) * 3 + which;
        if (at < 0 || at >= (int64_t)dir.size()) return false;
        switch (dir[at]) {
            case 1: --i; --j; which = 2; line -= width_d * 3; op = 'M'; break;
            case 2: --i; which = 0; line -= width_d * 3; op = 'I'; break;
            case 3: --i; which = 2; line -= width_d * 3; op = 'I'; break;
            case 4: --j; which = 1; op = 'D'; break;
            case 5: --j; which = 2; op = 'D'; break;
            default: return false;
        }
        if (op == prev) ++e;
        else {
            c.push_back(enc(e, prev));
            prev = op;
            e = 1;
        }
    }
    if (op == 'M') c.push_back(enc(e + 1, op));
    else {
        c.push_back(enc(e, op));
        c.push_back(enc(1, 'M'));
    }
    out.assign(c.rbegin(), c.rend());
    return true;
}

// ext/ssw/ssw.c:800-922 (ssw_init + ssw_align) with flag 0x0f, score filter 0 and
// distance filter INT32_MAX as src/ssw.rs:156-188 calls it (the suboptimal score
// is not used by the caller and is not computed).
SswResult ssw_align(const int8_t* read, int32_t read_len, const int8_t* ref, int32_t ref_len, const int8_t* mat,
                    int32_t n, uint8_t gap_open, uint8_t gap_extend) {
    SswResult r;
    int32_t bias = 0;
    for (int32_t i = 0; i < n * n; i++) bias = std::min<int32_t>(bias, mat[i]);
    bias = std::abs(bias);
    std::vector<uint8_t> pb = profile_byte(read, mat, read_len, n, (uint8_t)bias);
    EndPos best = sw_byte(ref, false, ref_len, read_len, gap_open, gap_extend, pb, 255, (uint8_t)bias);
    bool word = false;
    if (best.score == 255) {
        std::vector<int16_t> pw = profile_word(read, mat, read_len, n);
        best = sw_word(ref, false, ref_len, read_len, gap_open, gap_extend, pw, 65535);
        word = true;
    }
    r.score1 = best.score;
    r.ref_end1 = best.ref;
    r.read_end1 = best.read;
    std::vector<int8_t> rev(read, read + r.read_end1 + 1);
    std::reverse(rev.begin(), rev.end());
    EndPos back;
    if (!word) {
        std::vector<uint8_t> p = profile_byte(rev.data(), mat, r.read_end1 + 1, n, (uint8_t)bias);
        back = sw_byte(ref, true, r.ref_end1 + 1, r.read_end1 + 1, gap_open, gap_extend, p, (uint8_t)r.score1,
                       (uint8_t)bias);
    } else {
        std::vector<int16_t> p = profile_word(rev.data(), mat, r.read_end1 + 1, n);
        back = sw_word(ref, true, r.ref_end1 + 1, r.read_end1 + 1, gap_open, gap_extend, p, r.score1);
    }
    r.ref_begin1 = back.ref;
    r.read_begin1 = r.read_end1 - back.read;
    if (r.score1 > back.score) r.flag = 2;
    if (r.ref_begin1 < 0) return r;  // the caller discards this result (ref_begin1 == -1)
    int32_t rl = r.ref_end1 - r.ref_begin1 + 1, ql = r.read_end1 - r.read_begin1 + 1;
    if (!banded_sw(ref + r.ref_begin1, read + r.read_begin1, rl, ql, r.score1, gap_open, gap_extend,
                   std::abs(rl - ql) + 1, mat, n, r.cigar))
        r.flag = 1;
    return r;
}

// src/ssw.rs:8-25 (note: U/u translate to 0)
std::vector<int8_t> ssw_translate(const std::string& s) {
    std::vector<int8_t> t(s.size());
    for (size_t i = 0; i < s.size(); i++) {
        switch (s[i]) {
            case 'A': case 'a': case 'U': case 'u': t[i] = 0; break;
            case 'C': case 'c': t[i] = 1; break;
            case 'G': case 'g': t[i] = 2; break;
            case 'T': case 't': t[i] = 3; break;
            default: t[i] = 4;
        }
    }
    return t;
}

// src/ssw.rs:141-188 (SswAligner::new / align)
std::optional<AlignmentInfo> ssw_aligner_align(const std::string& query, const std::string& ref, const Scores& sc) {
    if (query.empty()) return std::nullopt;
    int8_t m = (int8_t)sc.match, x = (int8_t)-(int8_t)sc.mismatch;
    int8_t mat[25];
    for (int a = 0; a < 5; a++)
        for (int b = 0; b < 5; b++) mat[a * 5 + b] = (a == b && a < 4) ? m : x;
    std::vector<int8_t> tq = ssw_translate(query), tr = ssw_translate(ref);
    SswResult r = ssw_align(tq.data(), (int32_t)tq.size(), tr.data(), (int32_t)tr.size(), mat, 5, sc.gap_open,
                            sc.gap_extend);
    if (r.ref_begin1 == -1 || r.read_begin1 == -1) return std::nullopt;
    if (r.flag != 0) return std::nullopt;
    AlignmentInfo a;
    a.score = r.score1;
    a.ref_start = (size_t)r.ref_begin1;
    a.ref_end = (size_t)(r.ref_end1 + 1);
    a.query_start = (size_t)r.read_begin1;
    a.query_end = (size_t)(r.read_end1 + 1);
    Cigar raw;
    raw.ops = r.cigar;
    try {
        a.cigar = raw.with_eqx(query.substr(a.query_start, a.query_end - a.query_start),
                               ref.substr(a.ref_start, a.ref_end - a.ref_start));
    } catch (const std::out_of_range&) {
        return std::nullopt;  // the reference would panic here
    }
    a.edit_distance = a.cigar.edit_distance();
    return a;
}

// src/aligner.rs:80-151 (Aligner::align)
std::optional<AlignmentInfo> aligner_align(const std::string& query, const std::string& ref, const Scores& sc) {
    if (ref.size() > 2000) return std::nullopt;
    std::optional<AlignmentInfo> oa = ssw_aligner_align(query, ref, sc);
    if (!oa) return oa;
    AlignmentInfo& a = *oa;
    size_t qs = a.query_start, rs = a.ref_start;
    int32_t score = (int32_t)a.score;
    size_t edits = a.edit_distance;
    Cigar front;
    while (qs > 0 && rs > 0) {
        qs--;
        rs--;
        if (query[qs] == ref[rs]) { score += sc.match; front.push(OP_EQ, 1); }
        else { score -= sc.mismatch; front.push(OP_X, 1); edits++; }
    }
    int32_t swb = score + (int32_t)sc.end_bonus;
    if (qs == 0 && swb > (int32_t)a.score) {
        if (a.query_start > 0) {
            Cigar c = front.reversed();
            c.extend(a.cigar);
            a.cigar = c;
        }
        a.query_start = 0;
        a.ref_start = rs;
        a.score = (uint32_t)swb;
        a.edit_distance = edits;
    }
    size_t qe = a.query_end, re = a.ref_end;
    score = (int32_t)a.score;
    edits = a.edit_distance;
    Cigar back;
    while (qe < query.size() && re < ref.size()) {
        if (query[qe] == ref[re]) { score += sc.match; back.push(OP_EQ, 1); }
        else { score -= sc.mismatch; back.push(OP_X, 1); edits++; }
        qe++;
        re++;
    }
    swb = score + (int32_t)sc.end_bonus;
    if (qe == query.size() && swb > (int32_t)a.score) {
        if (a.query_end < query.size()) a.cigar.extend(back);
        a.query_end = query.size();
        a.ref_end = re;
        a.score = (uint32_t)swb;
        a.edit_distance = edits;
    }
    return oa;
}

// src/aligner.rs:181-216
void highest_scoring_segment(const std::string& q, const std::string& r, uint8_t match, uint8_t mismatch,
                             uint32_t end_bonus, size_t& bstart, size_t& bend, uint32_t& bscore) {
    size_t n = q.size(), start = 0;
    int32_t score = (int32_t)end_bonus, best = 0;
    bstart = 0;
    bend = 0;
    for (size_t i = 0; i < n; i++) {
        if (q[i] == r[i]) score += match;
        else score -= mismatch;
        if (score < 0) { start = i + 1; score = 0; }
        if (score > best) { bstart = start; best = score; bend = i + 1; }
    }
    if (score + (int32_t)end_bonus > best) {
        best = score + (int32_t)end_bonus;
        bend = q.size();
        bstart = start;
    }
    bscore = (uint32_t)best;
}

// src/aligner.rs:220-259
std::optional<AlignmentInfo> hamming_align(const std::string& q, const std::string& r, uint8_t match,
                                           uint8_t mismatch, uint32_t end_bonus) {
    if (q.size() != r.size()) return std::nullopt;
    size_t s, e;
    uint32_t score;
    highest_scoring_segment(q, r, match, mismatch, end_bonus, s, e, score);
    AlignmentInfo a;
    size_t mm = 0;
    for (size_t i = s; i < e; i++) {
        if (q[i] != r[i]) { mm++; a.cigar.push(OP_X, 1); }
        else a.cigar.push(OP_EQ, 1);
    }
    a.score = score;
    a.edit_distance = mm;
    a.ref_start = s;
    a.ref_end = e;
    a.query_start = s;
    a.query_end = e;
    return a;
}

// src/aligner.rs:261-291
AlignmentInfo hamming_align_global(const std::string& q, const std::string& r, uint8_t match, uint8_t mismatch) {
    AlignmentInfo a;
    int32_t score = 0;
    size_t n = std::min(q.size(), r.size());
    for (size_t i = 0; i < n; i++) {
        if (q[i] == r[i]) { score += match; a.cigar.push(OP_EQ, 1); }
        else { score -= mismatch; a.edit_distance++; a.cigar.push(OP_X, 1); }
    }
    a.ref_start = 0;
    a.ref_end = q.size();
    a.query_start = 0;
    a.query_end = q.size();
    a.score = (uint32_t)std::max(0, score);
    return a;
}

}  // namespace oracle
