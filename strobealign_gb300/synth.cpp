// Seeded synthetic genomes and reads with the shapes of the benchmark workloads
// (workload generator for the benchmark and the tests; not part of the mapping
// library).  Every random draw comes from xoshiro256** streams seeded by splitmix64
// from (seed, block), so the output depends only on the arguments, not on the thread
// count or the machine: integer arithmetic only, plus IEEE double additions and
// multiplications (no libm calls).
//
// Genome: contigs of total/n bases (+1 for the first total%n), bases drawn with the
// given GC content; then segmental duplications (copies of segdup_len bases between
// contigs at segdup_div substitutions), interspersed repeats (50 families of
// fam_lo..fam_hi bases, copies at a divergence uniform in [div_lo, div_hi] until
// repeat_fraction of the genome is covered) and tandem repeats (units of 2-50
// bases repeated over 100-3000 bases at 2% substitutions, tandem_fraction of the
// genome), applied in that order.
//
// Reads: single-end reads of a length uniform in [len_lo, len_hi], or FR pairs of
// len_lo bases from fragments of insert ~ Normal(insert_mean, insert_sd) (at least
// the read length; Irwin-Hall approximation), from uniform positions on both
// strands; substitutions at `sub` per base, insertions/deletions of 1-3 bases
// (geometric, p = 1/2, truncated) at `indel` per base, the read cut back to its
// length; a `rescue_fraction` of pairs has one mate with 15% extra substitutions.
#include <string>
#include <cstdio>
#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

namespace {

uint64_t splitmix(uint64_t& x) {
    uint64_t z = (x += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

struct Rng {
    uint64_t s[4];
    Rng(uint64_t seed, uint64_t stream) {
        uint64_t x = seed * 0x632BE59BD9B4E019ULL + stream * 0xD1342543DE82EF95ULL + 1;
        for (auto& v : s) v = splitmix(x);
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next() {
        uint64_t r = rotl(s[1] * 5, 7) * 9, t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return r;
    }
    double unit() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }  // [0, 1)
    uint64_t below(uint64_t n) { return n ? (uint64_t)(((unsigned __int128)next() * n) >> 64) : 0; }
    uint64_t range(uint64_t lo, uint64_t hi) { return lo + below(hi - lo + 1); }  // [lo, hi]
    bool chance(uint64_t thresh) { return next() < thresh; }                     // thresh = p * 2^64
    double normal() {  // Irwin-Hall(12) - 6
        double s = 0;
        for (int i = 0; i < 12; i++) s += unit();
        return s - 6.0;
    }
};

uint64_t threshold(double p) {
    if (p <= 0) return 0;
    if (p >= 1) return UINT64_MAX;
    return (uint64_t)(p * 18446744073709551616.0);
}

const uint8_t ACGT[4] = {'A', 'C', 'G', 'T'};

int code(uint8_t c) {
    switch (c) {
        case 'A': return 0;
        case 'C': return 1;
        case 'G': return 2;
        case 'T': return 3;
        default: return -1;
    }
}

uint8_t comp(uint8_t c) {
    switch (c) {
        case 'A': return 'T';
        case 'C': return 'G';
        case 'G': return 'C';
        case 'T': return 'A';
        default: return 'N';
    }
}

struct GcTable {
    uint64_t t0, t1, t2;  // cumulative thresholds of A, C, G over 2^16
    explicit GcTable(double gc) {
        double a = (1 - gc) / 2, c = gc / 2;
        t0 = (uint64_t)(a * 65536.0);
        t1 = (uint64_t)((a + c) * 65536.0);
        t2 = (uint64_t)((a + 2 * c) * 65536.0);
    }
    uint8_t base(uint64_t u16) const { return ACGT[(u16 >= t0) + (u16 >= t1) + (u16 >= t2)]; }
};

void random_bases(Rng& r, const GcTable& g, uint8_t* out, uint64_t n) {
    uint64_t i = 0;
    for (; i + 4 <= n; i += 4) {
        uint64_t x = r.next();
        for (int k = 0; k < 4; k++) out[i + k] = g.base((x >> (16 * k)) & 0xFFFF);
    }
    if (i < n) {
        uint64_t x = r.next();
        for (int k = 0; i < n; i++, k++) out[i] = g.base((x >> (16 * k)) & 0xFFFF);
    }
}

// each base with probability p becomes one of the three other bases
void mutate(Rng& r, uint8_t* a, uint64_t n, uint64_t thresh) {
    if (!thresh) return;
    for (uint64_t i = 0; i < n; i++)
        if (r.chance(thresh)) {
            int c = code(a[i]);
            if (c >= 0) a[i] = ACGT[(c + 1 + (int)r.below(3)) & 3];
        }
}

template <class F>
void parallel_for(uint64_t n, int threads, F f) {
    if (threads <= 1 || n <= 1) {
        for (uint64_t i = 0; i < n; i++) f(i);
        return;
    }
    std::atomic<uint64_t> next{0};
    std::vector<std::thread> th;
    for (int t = 0; t < threads; t++)
        th.emplace_back([&] {
            for (uint64_t i; (i = next.fetch_add(1)) < n;) f(i);
        });
    for (auto& t : th) t.join();
}

struct RepeatEvent {
    uint32_t family;
    uint64_t pos;
    uint64_t thresh;
    uint64_t stream;
};
struct TandemEvent {
    uint32_t period, length;
    uint64_t pos;
    uint64_t stream;
};

// one read (or mate) with substitutions and indels, cut back to len
void finish_read(Rng& r, std::vector<uint8_t>& s, uint64_t sub_t, uint64_t indel_t, uint64_t heavy_t,
                 std::vector<uint8_t>& tmp) {
    size_t len = s.size();
    mutate(r, s.data(), len, sub_t);
    if (heavy_t) mutate(r, s.data(), len, heavy_t);
    if (!indel_t) return;
    tmp.clear();
    size_t i = 0;
    bool any = false;
    while (i < len) {
        if (r.chance(indel_t)) {
            any = true;
            uint32_t L = 1;
            while (L < 3 && (r.next() >> 63)) L++;  // geometric(1/2) truncated at 3
            if (r.next() >> 63) {
                for (uint32_t k = 0; k < L; k++) tmp.push_back(ACGT[r.below(4)]);
                tmp.push_back(s[i++]);
            } else {
                i += L;
            }
        } else {
            tmp.push_back(s[i++]);
        }
    }
    if (!any) return;
    if (tmp.size() > len) tmp.resize(len);
    s.swap(tmp);
}

}  // namespace

extern "C" {

// Contig c spans [starts[c], starts[c+1]) of out (total bytes).
int32_t syn_genome(uint64_t seed, uint64_t total, uint32_t n_contigs, double gc, double segdup_fraction,
                   uint32_t segdup_len, double segdup_div, double repeat_fraction, uint32_t fam_lo, uint32_t fam_hi,
                   double div_lo, double div_hi, double tandem_fraction, uint8_t* out, int32_t threads) {
    if (!n_contigs || !out) return -1;
    std::vector<uint64_t> lens(n_contigs, total / n_contigs), starts(n_contigs + 1, 0);
    for (uint64_t i = 0; i < total % n_contigs; i++) lens[i]++;
    for (uint32_t c = 0; c < n_contigs; c++) starts[c + 1] = starts[c] + lens[c];
    GcTable g(gc);
    // bases: one stream per 1 Mbp block
    const uint64_t B = 1 << 20;
    parallel_for((total + B - 1) / B, threads, [&](uint64_t b) {
        Rng r(seed, 1000000 + b);
        random_bases(r, g, out + b * B, std::min(B, total - b * B));
    });
    Rng m(seed, 0);  // master stream: events in order
    // segmental duplications, sequential (a copy may read an earlier copy)
    uint64_t n_dup = segdup_len ? (uint64_t)((double)total * segdup_fraction / segdup_len) : 0;
    uint64_t dup_t = threshold(segdup_div);
    for (uint64_t i = 0; i < n_dup; i++) {
        uint32_t a = (uint32_t)m.below(n_contigs), b = (uint32_t)m.below(n_contigs);
        if (lens[a] <= segdup_len || lens[b] <= segdup_len) continue;
        uint64_t src = m.below(lens[a] - segdup_len), dst = m.below(lens[b] - segdup_len);
        std::memmove(out + starts[b] + dst, out + starts[a] + src, segdup_len);
        mutate(m, out + starts[b] + dst, segdup_len, dup_t);
    }
    // interspersed repeat families and tandem repeats: events drawn in order from
    // the master stream, applied per contig (in event order) in parallel
    std::vector<std::vector<uint8_t>> fams;
    std::vector<std::vector<RepeatEvent>> rep(n_contigs);
    std::vector<std::vector<TandemEvent>> tan(n_contigs);
    uint64_t stream = 1;
    if (repeat_fraction > 0) {
        for (int f = 0; f < 50; f++) {
            fams.emplace_back(m.range(fam_lo, fam_hi));
            random_bases(m, g, fams.back().data(), fams.back().size());
        }
        int64_t budget = (int64_t)((double)total * repeat_fraction);
        uint64_t guard = 0;
        while (budget > 0 && guard++ < (1ULL << 32)) {
            uint32_t f = (uint32_t)m.below(fams.size());
            uint32_t c = (uint32_t)m.below(n_contigs);
            uint64_t L = fams[f].size();
            if (lens[c] <= L) continue;
            uint64_t d = m.below(lens[c] - L);
            double div = div_lo + (div_hi - div_lo) * m.unit();
            rep[c].push_back({f, d, threshold(div), stream++});
            budget -= (int64_t)L;
        }
    }
    if (tandem_fraction > 0) {
        int64_t budget = (int64_t)((double)total * tandem_fraction);
        uint64_t guard = 0;
        while (budget > 0 && guard++ < (1ULL << 32)) {
            uint32_t period = (uint32_t)m.range(2, 50);
            uint32_t length = (uint32_t)m.range(100, 2999);
            uint32_t c = (uint32_t)m.below(n_contigs);
            if (lens[c] <= length) continue;
            uint64_t d = m.below(lens[c] - length);
            tan[c].push_back({period, length, d, stream++});
            budget -= (int64_t)length;
        }
    }
    const uint64_t tan_t = threshold(0.02);
    parallel_for(n_contigs, threads, [&](uint64_t c) {
        uint8_t* base = out + starts[c];
        for (const RepeatEvent& e : rep[c]) {
            Rng r(seed, e.stream);
            const std::vector<uint8_t>& f = fams[e.family];
            std::memcpy(base + e.pos, f.data(), f.size());
            mutate(r, base + e.pos, f.size(), e.thresh);
        }
        for (const TandemEvent& e : tan[c]) {
            Rng r(seed, e.stream);
            uint8_t unit[64];
            random_bases(r, g, unit, e.period);
            for (uint32_t i = 0; i < e.length; i++) base[e.pos + i] = unit[i % e.period];
            mutate(r, base + e.pos, e.length, tan_t);
        }
    });
    return 0;
}

// Reads from genome (contig c = [starts[c], starts[c+1])).  seq1/seq2 hold at least
// n * len_hi bytes, off1/off2 and name_off n + 1 entries, names n * 24 bytes.
// Read i (pair i) is named prefix + decimal i; mates share the name.  seq2/off2 NULL
// for single-end reads.  Returns 0.
int32_t syn_reads(uint64_t seed, const uint8_t* genome, const uint64_t* starts, uint32_t n_contigs, uint64_t n,
                  uint32_t len_lo, uint32_t len_hi, double insert_mean, double insert_sd, double sub, double indel,
                  double rescue_fraction, char prefix, uint8_t* seq1, uint64_t* off1, uint8_t* seq2, uint64_t* off2,
                  char* names, uint64_t* name_off, int32_t threads) {
    if (!n_contigs || !genome) return -1;
    const bool paired = seq2 != nullptr;
    const uint64_t total = starts[n_contigs];
    const uint64_t sub_t = threshold(sub), indel_t = threshold(indel), heavy_t = threshold(0.15);
    const uint64_t resc_t = threshold(rescue_fraction);
    const uint64_t BLK = 1 << 15;
    const uint64_t nb = (n + BLK - 1) / BLK;
    std::vector<std::vector<uint8_t>> out1(nb), out2(nb);
    std::vector<uint32_t> len1(n), len2(paired ? n : 0);
    auto pick = [&](Rng& r, uint64_t frag, uint64_t& pos, uint64_t& flen) {
        uint64_t u = r.below(total);
        uint32_t c = (uint32_t)(std::upper_bound(starts, starts + n_contigs + 1, u) - starts - 1);
        uint64_t L = starts[c + 1] - starts[c];
        uint64_t room = L > frag ? L - frag : 1;
        pos = starts[c] + (uint64_t)(r.unit() * (double)room);
        flen = std::min(frag, L);
    };
    parallel_for(nb, threads, [&](uint64_t b) {
        Rng r(seed, b);
        std::vector<uint8_t> s1, s2, tmp;
        uint64_t first = b * BLK, last = std::min(n, first + BLK);
        for (uint64_t i = first; i < last; i++) {
            if (!paired) {
                uint64_t L = r.range(len_lo, len_hi), pos, fl;
                pick(r, L, pos, fl);
                bool flip = r.next() >> 63;
                s1.resize(fl);
                for (uint64_t j = 0; j < fl; j++)
                    s1[j] = flip ? comp(genome[pos + fl - 1 - j]) : genome[pos + j];
                finish_read(r, s1, sub_t, indel_t, 0, tmp);
                len1[i] = (uint32_t)s1.size();
                out1[b].insert(out1[b].end(), s1.begin(), s1.end());
                continue;
            }
            const uint64_t length = len_lo;
            double x = insert_mean + insert_sd * r.normal();
            int64_t ins = (int64_t)(x < 0 ? x - 0.5 : x + 0.5);
            if (ins < (int64_t)length) ins = (int64_t)length;
            uint64_t pos, frag;
            pick(r, (uint64_t)ins, pos, frag);
            bool flip = r.next() >> 63;
            uint64_t L = std::min<uint64_t>(frag, length);
            s1.resize(L);
            s2.resize(L);
            for (uint64_t j = 0; j < L; j++) {
                uint8_t head = genome[pos + std::min(j, frag - 1)];
                uint8_t tail = comp(genome[pos + (frag - 1 >= j ? frag - 1 - j : 0)]);
                s1[j] = flip ? tail : head;
                s2[j] = flip ? head : tail;
            }
            bool heavy = resc_t && r.chance(resc_t);
            bool which = r.next() >> 63;
            finish_read(r, s1, sub_t, indel_t, heavy && which ? heavy_t : 0, tmp);
            finish_read(r, s2, sub_t, indel_t, heavy && !which ? heavy_t : 0, tmp);
            len1[i] = (uint32_t)s1.size();
            len2[i] = (uint32_t)s2.size();
            out1[b].insert(out1[b].end(), s1.begin(), s1.end());
            out2[b].insert(out2[b].end(), s2.begin(), s2.end());
        }
    });
    // offsets, then the blocks copied into place in parallel
    std::vector<uint64_t> bo1(nb + 1, 0), bo2(nb + 1, 0), bno(nb + 1, 0);
    off1[0] = 0;
    if (paired) off2[0] = 0;
    name_off[0] = 0;
    for (uint64_t i = 0; i < n; i++) {
        off1[i + 1] = off1[i] + len1[i];
        if (paired) off2[i + 1] = off2[i] + len2[i];
        uint64_t digits = 1;
        for (uint64_t v = i; v >= 10; v /= 10) digits++;
        name_off[i + 1] = name_off[i] + 1 + digits;
    }
    parallel_for(nb, threads, [&](uint64_t b) {
        uint64_t first = b * BLK, last = std::min(n, first + BLK);
        std::memcpy(seq1 + off1[first], out1[b].data(), out1[b].size());
        if (paired) std::memcpy(seq2 + off2[first], out2[b].data(), out2[b].size());
        for (uint64_t i = first; i < last; i++) {
            char* p = names + name_off[i];
            *p++ = prefix;
            char buf[24];
            int k = 0;
            uint64_t v = i;
            do {
                buf[k++] = (char)('0' + v % 10);
                v /= 10;
            } while (v);
            while (k) *p++ = buf[--k];
        }
        std::vector<uint8_t>().swap(out1[b]);
        if (paired) std::vector<uint8_t>().swap(out2[b]);
    });
    return 0;
}

// Records [0, n) as FASTQ ("@name", sequence, "+", quality; qual NULL writes 'I' for
// every base) to path; 0 on success, -1 on an I/O error.
int32_t syn_write_fastq(const char* path, uint64_t n, const uint8_t* seq, const uint64_t* off, const uint8_t* names,
                        const uint64_t* name_off, const uint8_t* qual) {
    FILE* f = std::fopen(path, "wb");
    if (!f) return -1;
    std::vector<char> buf;
    buf.reserve((size_t)8 << 20);
    bool ok = true;
    std::string fill;
    for (uint64_t i = 0; i < n && ok; i++) {
        const uint64_t a = off[i], b = off[i + 1];
        buf.push_back('@');
        buf.insert(buf.end(), names + name_off[i], names + name_off[i + 1]);
        buf.push_back('\n');
        buf.insert(buf.end(), seq + a, seq + b);
        buf.insert(buf.end(), {'\n', '+', '\n'});
        if (qual) {
            buf.insert(buf.end(), qual + a, qual + b);
        } else {
            if (fill.size() < b - a) fill.assign(b - a, 'I');
            buf.insert(buf.end(), fill.begin(), fill.begin() + (ptrdiff_t)(b - a));
        }
        buf.push_back('\n');
        if (buf.size() >= ((size_t)8 << 20)) {
            ok = std::fwrite(buf.data(), 1, buf.size(), f) == buf.size();
            buf.clear();
        }
    }
    if (ok && !buf.empty()) ok = std::fwrite(buf.data(), 1, buf.size(), f) == buf.size();
    if (std::fclose(f) != 0) ok = false;
    return ok ? 0 : -1;
}

}  // extern "C"
