// The GPU striped Smith-Waterman (strobealign_gb300/csrc/extend.cu, k_ssw and
// k_ssw_wave) computes
// two parts of ssw.c's striped passes (ext/ssw/ssw.c:163-596) in a different form:
//   * the in-segment F recurrence as vF' = max(vF - gE, max(max(vH + m, E) - gO, 0)),
//   * the lazy-F loop (ext/ssw/ssw.c:285-299) in closed form:
//     H(l, j) = max(H, G(l) - j*gE), G(l) = max over lanes l' < l of
//     Ffinal(l') - (l - 1 - l') * segLen * gE.
// This program runs both the library's order of operations (mode 0) and the
// rewritten form (mode 2) on random tasks with planted alignments and compares
// every column's H and E and the reported maximum and end positions.  Valid for
// gap_open > gap_extend, the case the GPU kernels are used for (with equal penalties
// the library's lazy-F loop stops after the first row of each lane).
// Usage: ssw_reformulation_check [trials]; exit status 1 on any difference.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
static unsigned long long rs = 88172645463325252ULL;  // xorshift64 state
static unsigned rnd(void) { rs ^= rs << 13; rs ^= rs >> 7; rs ^= rs << 17; return (unsigned)rs; }
static int mx(int a, int b) { return a > b ? a : b; }
// one striped pass; mode 0 = original lazy-F, 1 = closed form. returns checksum of per-column H/E and max info
static long run(const int* q, int qlen, const int* r, int rlen, int NL, int gO, int gE, int match, int mism, int mode,
                int* Hout, int* Eout) {
    int seg = (qlen + NL - 1) / NL;
    int n = seg * NL;
    int* H = calloc(n, sizeof(int)); int* E = calloc(n, sizeof(int));
    int* prof = malloc(sizeof(int) * n);
    long chk = 0;
    int maxv = 0, end_ref = -1, end_read = qlen - 1;
    for (int i = 0; i < rlen; i++) {
        int rb = r[i];
        for (int l = 0; l < NL; l++) for (int j = 0; j < seg; j++) {
            int pos = l * seg + j;
            prof[l * seg + j] = pos < qlen ? ((q[pos] == rb && rb < 4) ? match : -mism) : 0;
        }
        // main loop, all lanes
        int vFfinal[64];
        int vMaxCol = 0;
        for (int l = 0; l < NL; l++) {
            int vH = l == 0 ? 0 : H[(l - 1) * seg + seg - 1];
            int vF = 0;
            for (int j = 0; j < seg; j++) {
                int idx = l * seg + j;
                int h = mx(vH + prof[idx], 0);
                int e = E[idx];
                if (mode == 2) {
                    int A = mx(h, e);
                    int a = mx(A - gO, 0);
                    h = mx(A, vF);
                    vMaxCol = mx(vMaxCol, h);
                    vH = H[idx];
                    H[idx] = h;
                    int hg = mx(h - gO, 0);
                    E[idx] = mx(e - gE, hg);
                    vF = mx(vF - gE, a);
                    continue;
                }
                h = mx(h, e); h = mx(h, vF);
                vMaxCol = mx(vMaxCol, h);
                vH = H[idx];  // old value (main loop reads stored H of prev column)
                H[idx] = h;
                int hg = mx(h - gO, 0);
                E[idx] = mx(mx(e - gE, 0), hg);
                vF = mx(mx(vF - gE, 0), hg);
            }
            vFfinal[l] = vF;
        }
        // NOTE vH above: diag for row j+1 is the previous column's H at row j; we overwrote H[idx]
        // after saving vH = old H[idx], correct.
        if (mode == 0) {
            int vF[64];
            for (int l = 0; l < NL; l++) vF[l] = vFfinal[l];
            for (int kk = 0; kk < NL; kk++) {
                for (int l = NL - 1; l > 0; l--) vF[l] = vF[l - 1];
                vF[0] = 0;
                int done = 0;
                for (int j = 0; j < seg; j++) {
                    int all = 1;
                    for (int l = 0; l < NL; l++) {
                        int idx = l * seg + j;
                        int h = mx(H[idx], vF[l]);
                        vMaxCol = mx(vMaxCol, h);
                        H[idx] = h;
                        int hg = mx(h - gO, 0);
                        vF[l] = mx(vF[l] - gE, 0);
                        if (vF[l] > hg) all = 0;
                    }
                    if (all) { done = 1; break; }
                }
                if (done) break;
            }
        } else {  /* modes 1, 2: closed form */
            int G = 0;  // exclusive scan over lanes
            for (int l = 0; l < NL; l++) {
                for (int j = 0; j < seg; j++) {
                    int idx = l * seg + j;
                    int h = mx(H[idx], G - j * gE);
                    vMaxCol = mx(vMaxCol, h);
                    H[idx] = h;
                }
                G = mx(G - seg * gE, vFfinal[l]);
            }
        }
        if (vMaxCol > maxv) {
            maxv = vMaxCol; end_ref = i;
            int best = 1 << 30;
            for (int l = 0; l < NL; l++) for (int j = 0; j < seg; j++) if (H[l * seg + j] == maxv && l * seg + j < best) best = l * seg + j;
            end_read = best < qlen - 1 ? best : qlen - 1;
        }
        for (int x = 0; x < n; x++) { Hout[(long)i * n + x] = H[x]; Eout[(long)i * n + x] = E[x]; }
    }
    chk = (long)maxv * 1000003 + end_ref * 1009 + end_read;
    free(H); free(E); free(prof);
    return chk;
}
int main(int argc, char** argv) {
    int trials = argc > 1 ? atoi(argv[1]) : 20000;
    int bad = 0; long cols = 0, lazylong = 0;
    int pens[][4] = {{12, 1, 2, 8}, {12, 1, 2, 8}, {6, 1, 1, 4}, {5, 2, 2, 3}, {11, 1, 1, 1}, {5, 4, 2, 2}, {3, 1, 5, 1}};
    for (int t = 0; t < trials; t++) {
        int* P = pens[rnd() % 7];
        int gO = P[0], gE = P[1], match = P[2], mism = P[3];
        int qlen = 1 + rnd() % 300;
        int NL = (rnd() & 1) ? 16 : 8;
        int q[400], r[2400];
        for (int i = 0; i < qlen; i++) q[i] = rnd() % 100 < 2 ? 4 : rnd() % 4;
        int rlen = 0;
        int pre = rnd() % 60;
        for (int i = 0; i < pre; i++) r[rlen++] = rnd() % 4;
        for (int i = 0; i < qlen && rlen < 2300; i++) {
            int x = rnd() % 1000;
            if (x < 20) r[rlen++] = rnd() % 4;
            else if (x < 30) {}
            else if (x < 40) { r[rlen++] = q[i]; int g = 1 + rnd() % 6; for (int k = 0; k < g; k++) r[rlen++] = rnd() % 4; }
            else if (x < 45) { i += rnd() % 6; }
            else r[rlen++] = q[i];
        }
        int post = rnd() % 60;
        for (int i = 0; i < post && rlen < 2390; i++) r[rlen++] = rnd() % 4;
        int seg = (qlen + NL - 1) / NL;
        int* H0 = malloc(sizeof(int) * (long)rlen * seg * NL); int* E0 = malloc(sizeof(int) * (long)rlen * seg * NL);
        int* H1 = malloc(sizeof(int) * (long)rlen * seg * NL); int* E1 = malloc(sizeof(int) * (long)rlen * seg * NL);
        long a = run(q, qlen, r, rlen, NL, gO, gE, match, mism, 0, H0, E0);
        long b = run(q, qlen, r, rlen, NL, gO, gE, match, mism, 2, H1, E1);
        cols += rlen;
        if (a != b || memcmp(H0, H1, sizeof(int) * (long)rlen * seg * NL) || memcmp(E0, E1, sizeof(int) * (long)rlen * seg * NL)) {
            bad++;
            if (bad < 5) printf("mismatch trial %d qlen %d rlen %d NL %d pens %d %d %d %d\n", t, qlen, rlen, NL, gO, gE, match, mism);
        }
        free(H0); free(E0); free(H1); free(E1);
    }
    printf("trials %d columns %ld mismatches %d\n", trials, cols, bad);
    return bad != 0;
}
