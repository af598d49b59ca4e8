// Oracle (test infrastructure only): command line driver.  Restates the parts of
// src/main.rs that fix output bytes: read-length estimation (:1003-1012), chunking
// (:591-604, chunk = records until the nucleotide count exceeds chunk_size), a fresh
// Rng::with_seed(0) and InsertSizeDistribution per chunk (:878-879), output in chunk
// order (:653-667) and the abundance table (:990-1001).  Chunks run on -t threads
// (driver.cpp), and so does the index build.  --interleaved pairs consecutive records
// of one file by name (src/io/reads.rs:68-113).
//
//   sa_oracle [options] ref.fa reads1.fq [reads2.fq]
#include "oracle.hpp"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <thread>

using namespace oracle;

namespace {

struct Args {
    size_t threads = 1, chunk_size = 1000000;
    bool map_only = false, aemb = false, eqx = false, no_pg = false, only_mapped = false, details = false;
    bool fastq_comments = false, use_ssw = false, interleaved = false;
    std::string rg_id;
    bool has_rg_id = false;
    std::vector<std::string> rg;
    size_t max_secondary = 0, read_length = 0, max_tries = 20, rescue_distance = 100;
    bool has_read_length = false;
    Mcs mcs = Mcs::Always;
    double filter_fraction = 0.0002;
    float dropoff = 0.5f;
    std::vector<std::string> pos;
    bool timing = false;
    std::string output;
};

bool parse(int argc, char** argv, Args& a, std::string& err) {
    for (int i = 1; i < argc; i++) {
        std::string s = argv[i];
        std::string key = s, val;
        bool has_val = false;
        size_t eq = s.find('=');
        if (s.rfind("--", 0) == 0 && eq != std::string::npos) {
            key = s.substr(0, eq);
            val = s.substr(eq + 1);
            has_val = true;
        }
        auto next = [&]() -> std::string {
            if (has_val) return val;
            if (i + 1 >= argc) { err = "missing value for " + key; return ""; }
            return argv[++i];
        };
        if (key == "-t") a.threads = std::stoul(next());
        else if (key == "--chunk-size") a.chunk_size = std::stoul(next());
        else if (key == "-x") a.map_only = true;
        else if (key == "--aemb") a.aemb = true;
        else if (key == "--eqx") a.eqx = true;
        else if (key == "--no-PG") a.no_pg = true;
        else if (key == "-U") a.only_mapped = true;
        else if (key == "--details") a.details = true;
        else if (key == "-C") a.fastq_comments = true;
        else if (key == "--ssw") a.use_ssw = true;
        else if (key == "--interleaved") a.interleaved = true;
        else if (key == "--rg-id") { a.rg_id = next(); a.has_rg_id = true; }
        else if (key == "--rg") a.rg.push_back(next());
        else if (key == "-N") a.max_secondary = std::stoul(next());
        else if (key == "-r") { a.read_length = std::stoul(next()); a.has_read_length = true; }
        else if (key == "-M") a.max_tries = std::stoul(next());
        else if (key == "-R") a.rescue_distance = std::stoul(next());
        else if (key == "-f") a.filter_fraction = std::stod(next());
        else if (key == "-S") a.dropoff = std::stof(next());
        else if (key == "--timing") a.timing = true;
        else if (key == "-o") a.output = next();
        else if (key == "--mcs") {
            std::string v = next();
            if (v == "always") a.mcs = Mcs::Always;
            else if (v == "rescue") a.mcs = Mcs::Rescue;
            else if (v == "off") a.mcs = Mcs::Off;
            else if (v == "first-strobe") a.mcs = Mcs::FirstStrobe;
            else { err = "bad --mcs " + v; return false; }
        } else if (!s.empty() && s[0] == '-' && s != "-") {
            err = "unknown option " + s;
            return false;
        } else {
            a.pos.push_back(s);
        }
        if (!err.empty()) return false;
    }
    if (a.pos.size() < 2) { err = "usage: sa_oracle [options] ref.fa reads1.fq [reads2.fq]"; return false; }
    return true;
}

}  // namespace

int main(int argc, char** argv) {
    Args a;
    std::string err;
    if (!parse(argc, argv, a, err)) {
        std::fprintf(stderr, "error: %s\n", err.c_str());
        return 2;
    }
    std::vector<RefSeq> refs;
    if (!read_fasta(a.pos[0], refs, err)) { std::fprintf(stderr, "error: %s\n", err.c_str()); return 1; }
    if (refs.empty()) { std::fprintf(stderr, "error: No sequences found in the reference FASTA\n"); return 1; }
    std::vector<SequenceRecord> r1, r2;
    if (!read_fastq_file(a.pos[1], r1, err)) { std::fprintf(stderr, "error: %s\n", err.c_str()); return 1; }
    if (a.interleaved && a.pos.size() > 2) { std::fprintf(stderr, "error: --interleaved takes one reads file\n"); return 2; }
    bool paired = a.pos.size() > 2 || a.interleaved;
    if (a.pos.size() > 2 && !read_fastq_file(a.pos[2], r2, err)) { std::fprintf(stderr, "error: %s\n", err.c_str()); return 1; }
    size_t read_length = a.read_length;
    if (!a.has_read_length) {
        // estimate_read_length over the first 500 records of the first file (src/main.rs:351)
        size_t s = 0, n = 0;
        for (size_t i = 0; i < r1.size() && i < 500; i++) { s += r1[i].seq.size(); n++; }
        read_length = n ? s / n : 0;
    }
    std::vector<uint8_t> has_mate;
    if (a.interleaved) {
        std::vector<SequenceRecord> flat;
        flat.swap(r1);
        pair_interleaved(std::move(flat), r1, r2, has_mate);
    }
    SeedingParameters sp = SeedingParameters::from_read_length(read_length);
    auto t0 = std::chrono::steady_clock::now();
    uint8_t bits = pick_bits(refs, sp);
    Index index = make_index(refs, sp, bits, a.filter_fraction, std::max<size_t>(a.threads, 1));
    auto t1 = std::chrono::steady_clock::now();

    Context ctx;
    ctx.refs = &refs;
    ctx.index = &index;
    ctx.mp.max_secondary = a.max_secondary;
    ctx.mp.dropoff_threshold = a.dropoff;
    ctx.mp.rescue_distance = a.rescue_distance;
    ctx.mp.max_tries = a.max_tries;
    ctx.mp.mcs = a.mcs;
    ctx.mp.output_unmapped = !a.only_mapped;
    ctx.mp.use_ssw = a.use_ssw;
    ctx.so.eqx = a.eqx;
    ctx.so.details = a.details;
    ctx.so.fastq_comments = a.fastq_comments;
    if (a.has_rg_id) { ctx.so.rg_id = a.rg_id; ctx.so.has_rg = true; }
    else if (!a.rg.empty()) { ctx.so.rg_id = "1"; ctx.so.has_rg = true; }

    MapMode mode = a.aemb ? MapMode::Abundance : a.map_only ? MapMode::Paf : MapMode::Sam;
    size_t nt = std::max<size_t>(a.threads, 1);
    size_t n = paired ? std::min(r1.size(), r2.size()) : r1.size();
    std::vector<double> tot;
    std::vector<std::string> outs = map_records(ctx, r1, paired ? &r2 : nullptr, mode, nt, a.chunk_size, &tot,
                                                a.interleaved ? &has_mate : nullptr);
    auto t2 = std::chrono::steady_clock::now();

    FILE* fo = a.output.empty() ? stdout : std::fopen(a.output.c_str(), "wb");
    if (!fo) { std::fprintf(stderr, "error: cannot open output\n"); return 1; }
    if (!a.map_only && !a.aemb) {
        std::string cmd;
        for (int i = 1; i < argc; i++) { if (i > 1) cmd += ' '; cmd += argv[i]; }
        const std::string* rg = ctx.so.has_rg ? &ctx.so.rg_id : nullptr;
        std::string h = sam_header(refs, a.no_pg ? nullptr : &cmd, "0.18.0-alpha", rg, a.rg);
        std::fwrite(h.data(), 1, h.size(), fo);
    }
    for (auto& o : outs) std::fwrite(o.data(), 1, o.size(), fo);
    if (a.aemb) {
        for (size_t i = 0; i < refs.size(); i++)
            std::fprintf(fo, "%s\t%.6f\n", refs[i].name.c_str(), tot[i] / (double)refs[i].seq.len);
    }
    if (fo != stdout) std::fclose(fo);
    if (a.timing) {
        double ti = std::chrono::duration<double>(t1 - t0).count();
        double tm = std::chrono::duration<double>(t2 - t1).count();
        std::fprintf(stderr, "oracle_timing index_s=%.6f map_s=%.6f reads=%zu threads=%zu\n", ti, tm,
                     a.interleaved ? n + (size_t)std::count(has_mate.begin(), has_mate.end(), 1) : paired ? 2 * n : n,
                     nt);
    }
    return 0;
}
