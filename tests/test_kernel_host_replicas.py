"""Host builds of device functions from strobealign_gb300/csrc/extend.cu, checked against
their literal forms on random inputs (no GPU): the thread-per-task banded pass against
the literal banded_sw pass (ext/ssw/ssw.c:614-676) -- maxima and every direction byte --
and the run-length =/X CIGAR of a match bit array against the per-base walk."""
import shutil
import subprocess

import pytest

from conftest import ROOT

SRC = ROOT / "strobealign_gb300" / "csrc" / "extend.cu"

PRELUDE = r"""
#include <cstdint>
#include <cstdio>
#include <random>
#include <vector>
#define __device__
#define __forceinline__ inline
struct AlignScores { uint8_t match, mismatch, gap_open, gap_extend; };
static int c_ssw_code[256];
static int __ffs(uint32_t x) { return x ? __builtin_ctz(x) + 1 : 0; }
"""

BAND_MAIN = r"""
template <int BW> static int thread_pass(const std::vector<uint8_t>& r, const std::vector<uint8_t>& q,
                                         std::vector<uint32_t>& rows) {
    uint64_t cells = 0;
    AlignScores sc{2, 8, 12, 1};
    return band_pass_thread<BW>(r.data(), q.data(), (int)r.size(), (int)q.size(), sc, rows.data(), cells);
}
int main() {
    for (int c = 0; c < 256; c++) c_ssw_code[c] = 4;
    c_ssw_code['A'] = 0; c_ssw_code['C'] = 1; c_ssw_code['G'] = 2; c_ssw_code['T'] = 3;
    std::mt19937 rng(7);
    AlignScores sc{2, 8, 12, 1};
    long bad = 0, total = 0;
    for (int it = 0; it < 40000; it++) {
        int ql = 1 + rng() % 60, rl = 1 + rng() % 60;
        if (rng() % 2) { rl = ql + (int)(rng() % 5) - 2; if (rl < 1) rl = 1; }
        std::vector<uint8_t> q(ql), r(rl);
        const char* A = "ACGTN";
        for (auto& x : q) x = A[rng() % (rng() % 20 == 0 ? 5 : 4)];
        for (int i = 0; i < rl; i++) r[i] = (i < ql && rng() % 10) ? q[i] : A[rng() % 4];
        for (int bw = 1; bw <= 5; bw++) {
            const int width = 2 * bw + 3, wd = 2 * bw + 1;
            std::vector<int> hb(width + 2), eb(width + 2), hc(width + 2);
            std::vector<uint8_t> dir((size_t)wd * ql * 3, 0);
            const int m1 = band_pass(r.data(), q.data(), rl, ql, bw, sc, hb.data(), eb.data(), hc.data(), dir.data());
            std::vector<uint32_t> rows(2 * ql);
            int m2 = bw == 1 ? thread_pass<1>(r, q, rows) : bw == 2 ? thread_pass<2>(r, q, rows)
                   : bw == 3 ? thread_pass<3>(r, q, rows) : bw == 4 ? thread_pass<4>(r, q, rows) : thread_pass<5>(r, q, rows);
            total++;
            bool ok = m1 == m2;
            for (int i = 0; i < ql && ok; i++) {
                const int x = i - bw > 0 ? i - bw : 0, end = rl - 1 < i + bw ? rl - 1 : i + bw;
                for (int k = 0; k <= end - x; k++) {
                    const uint8_t de = dir[(size_t)wd * i * 3 + k * 3], df = dir[(size_t)wd * i * 3 + k * 3 + 1],
                                  dh = dir[(size_t)wd * i * 3 + k * 3 + 2];
                    const uint32_t a = rows[2 * i], b = rows[2 * i + 1];
                    const int dde = (a >> k) & 1 ? 3 : 2, ddf = (a >> (16 + k)) & 1 ? 5 : 4;
                    const int dhh = (b >> k) & 1 ? 1 : (((b >> (16 + k)) & 1) ? dde : ddf);
                    if (de != dde || df != ddf || dh != dhh) { ok = false; break; }
                }
            }
            bad += !ok;
        }
    }
    printf("%ld %ld\n", total, bad);
    return bad != 0;
}
"""

CIGAR_MAIN = r"""
int main() {
    std::mt19937 rng(3);
    long bad = 0, total = 0;
    for (int it = 0; it < 100000; it++) {
        const int L = 1 + rng() % 300;
        std::vector<uint32_t> bits((L + 31) / 32 + 1, 0);
        const int mode = rng() % 3;
        for (int i = 0; i < L; i++) {
            const bool e = mode == 0 ? rng() % 2 : mode == 1 ? (rng() % 20 != 0) : (rng() % 3 != 0);
            if (e) bits[i >> 5] |= 1u << (i & 31);
        }
        if (L % 32) bits[L >> 5] |= (rng() & ~((1u << (L % 32)) - 1));
        const uint32_t bs = rng() % (L + 1), be = bs + rng() % (L - bs + 1);
        std::vector<uint32_t> o1(2 * L + 8), o2(2 * L + 8);
        CigarWriter w1{o1.data(), 0, (uint32_t)o1.size(), false}, w2{o2.data(), 0, (uint32_t)o2.size(), false};
        auto eq = [&](uint32_t i) { return (bool)((bits[i >> 5] >> (i & 31)) & 1); };
        const uint32_t m1 = hamming_cigar(eq, bs, be, w1), m2 = hamming_cigar_bits(bits.data(), bs, be, w2);
        bool ok = m1 == m2 && w1.n == w2.n && w1.overflow == w2.overflow;
        for (uint32_t k = 0; ok && k < w1.n; k++) ok = o1[k] == o2[k];
        total++;
        bad += !ok;
    }
    printf("%ld %ld\n", total, bad);
    return bad != 0;
}
"""


def _grab(text: str, start: str, end: str = "\n}\n") -> str:
    a = text.index(start)
    return text[a:text.index(end, a) + len(end)]


def _run(tmp_path, name, body):
    if not shutil.which("g++"):
        pytest.skip("no g++")
    src = tmp_path / f"{name}.cpp"
    src.write_text(body)
    exe = tmp_path / name
    subprocess.run(["g++", "-O2", "-std=c++17", "-o", str(exe), str(src)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    total, bad = map(int, out.stdout.split())
    assert out.returncode == 0 and bad == 0 and total > 0, out.stdout


def test_thread_band_pass_matches_literal_pass(tmp_path):
    s = SRC.read_text()
    body = (PRELUDE + _grab(s, "__device__ __forceinline__ int mat_score(") +
            _grab(s, "__device__ int band_pass(const uint8_t* ref") +
            _grab(s, "template <int BW>\n__device__ int band_pass_thread(") + BAND_MAIN)
    _run(tmp_path, "band", body)


def test_run_length_hamming_cigar_matches_per_base_walk(tmp_path):
    s = SRC.read_text()
    body = (PRELUDE + _grab(s, "struct CigarWriter {", "\n};\n") +
            _grab(s, "template <class EQ>\n__device__ __forceinline__ uint32_t hamming_cigar(") +
            _grab(s, "__device__ __forceinline__ uint32_t hamming_cigar_bits(") + CIGAR_MAIN)
    _run(tmp_path, "cigar", body)
