// Host-side inputs: reference contigs (2-bit PackedSeq form) and read batches.
// FASTA: src/io/fasta.rs:116-165; FASTQ: src/io/fastq.rs:19-100; headers split
// as src/io/mod.rs:33-40; wildcard bases encoded as src/packed_seq.rs:50-92.
#include "host_state.h"

#include <cmath>
#include <cstring>
#include <fstream>

namespace sa {

static std::string trim_end(const std::string& s) {
    size_t e = s.size();
    while (e > 0 && (s[e - 1] == ' ' || s[e - 1] == '\t' || s[e - 1] == '\n' || s[e - 1] == '\r' ||
                     s[e - 1] == '\f' || s[e - 1] == '\v'))
        e--;
    return s.substr(0, e);
}

static void split_header(const std::string& h, std::string& name, std::string& comment, bool& has_comment) {
    std::string t = trim_end(h);
    size_t p = t.find_first_of(" \t");
    if (p == std::string::npos) {
        name = t;
        comment.clear();
        has_comment = false;
    } else {
        name = t.substr(0, p);
        comment = t.substr(p + 1);
        has_comment = true;
    }
}

void Contig::push(uint8_t c) {
    uint64_t v;
    switch (c) {
        case 'A': case 'a': v = 0; break;
        case 'C': case 'c': v = 1; break;
        case 'G': case 'g': v = 2; break;
        case 'T': case 't': case 'U': case 'u': v = 3; break;
        default: {
            uint64_t h = (uint64_t)len * 0x9e3779b97f4a7c15ULL;
            v = (h ^ (h >> 30)) & 3;
        }
    }
    size_t bit = (len & 31) * 2;
    if (bit == 0) words.push_back(v);
    else words.back() |= v << bit;
    len++;
}

static void validate_names(const std::vector<Contig>& cs) {
    std::vector<const std::string*> names;
    for (auto& c : cs) {
        if (c.name.empty()) throw Error(SA_ERR_FORMAT, "Invalid character in record name");
        for (unsigned char ch : c.name)
            if (ch < 33 || ch > 126) throw Error(SA_ERR_FORMAT, "Invalid character in record name");
        names.push_back(&c.name);
    }
    std::sort(names.begin(), names.end(), [](auto a, auto b) { return *a < *b; });
    for (size_t i = 1; i < names.size(); i++)
        if (*names[i] == *names[i - 1]) throw Error(SA_ERR_FORMAT, "Duplicate record name " + *names[i]);
}

void load_fasta(const std::string& path, std::vector<Contig>& out) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw Error(SA_ERR_IO, "cannot open " + path);
    std::string line;
    bool have = false;
    Contig cur;
    while (std::getline(f, line)) {
        if (!line.empty() && line[0] == '>') {
            if (have) out.push_back(std::move(cur));
            cur = Contig();
            std::string c;
            bool hc;
            split_header(line.substr(1), cur.name, c, hc);
            have = true;
        } else if (have) {
            std::string t = trim_end(line);
            for (char ch : t) cur.push((uint8_t)ch);
        } else if (!trim_end(line).empty()) {
            throw Error(SA_ERR_FORMAT, "FASTA file must start with '>'");
        }
    }
    if (have) out.push_back(std::move(cur));
    validate_names(out);
}

void contigs_from_buffers(size_t n, const char* const* names, const char* const* seqs, const size_t* lens,
                          std::vector<Contig>& out) {
    out.resize(n);
    for (size_t i = 0; i < n; i++) {
        out[i].name = names[i];
        out[i].words.reserve(lens[i] / 32 + 1);
        for (size_t j = 0; j < lens[i]; j++) out[i].push((uint8_t)seqs[i][j]);
    }
    validate_names(out);
}

// src/indexer.rs:294-300
uint32_t pick_bits(const std::vector<Contig>& cs, const SeedParams& p) {
    size_t total = 0;
    for (auto& c : cs) total += c.len;
    size_t est = total / (p.k - p.s + 1) + 1;
    uint32_t lg = (uint32_t)std::log2((double)est);
    if (lg < 9) lg = 9;
    if (lg > 32) lg = 32;
    return lg - 1;
}

static void push_str(std::string& buf, std::vector<uint64_t>& off, const std::string& s) {
    buf += s;
    off.push_back(buf.size());
}

void load_reads(const std::string& path, ReadStore& rs) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw Error(SA_ERR_IO, "cannot open " + path);
    rs = ReadStore();
    rs.seq_off.push_back(0);
    rs.name_off.push_back(0);
    rs.comment_off.push_back(0);
    int first = f.peek();
    if (first == '>') {
        std::string line, name, comment, seq;
        bool have = false, hc = false;
        auto flush = [&]() {
            push_str(rs.seq, rs.seq_off, seq);
            push_str(rs.names, rs.name_off, name);
            push_str(rs.comments, rs.comment_off, hc ? comment : std::string());
            rs.has_comment.push_back(hc);
            seq.clear();
        };
        while (std::getline(f, line)) {
            if (!line.empty() && line[0] == '>') {
                if (have) flush();
                split_header(line.substr(1), name, comment, hc);
                have = true;
            } else {
                std::string t = trim_end(line);
                for (char& c : t) c = (char)toupper((unsigned char)c);
                seq += t;
            }
        }
        if (have) flush();
        rs.has_qual = false;
        return;
    }
    rs.has_qual = true;
    rs.qual_off_unused = 0;
    std::string l1, l2, l3, l4, name, comment;
    bool hc;
    while (std::getline(f, l1)) {
        if (l1.empty() || l1[0] != '@') throw Error(SA_ERR_FORMAT, "FASTQ record must start with '@'");
        split_header(l1.substr(1), name, comment, hc);
        if (name.empty()) throw Error(SA_ERR_FORMAT, "Record identifier is empty");
        if (name.size() >= 2 && (name.compare(name.size() - 2, 2, "/1") == 0 || name.compare(name.size() - 2, 2, "/2") == 0))
            name.resize(name.size() - 2);
        std::getline(f, l2);
        std::getline(f, l3);
        std::getline(f, l4);
        if (!l2.empty() && l2.back() == '\r') l2.pop_back();
        if (!l4.empty() && l4.back() == '\r') l4.pop_back();
        if (l2.size() != l4.size()) throw Error(SA_ERR_FORMAT, "sequence and quality lengths differ in " + name);
        for (char& c : l2) c = (char)toupper((unsigned char)c);
        push_str(rs.seq, rs.seq_off, l2);
        rs.qual += l4;
        push_str(rs.names, rs.name_off, name);
        push_str(rs.comments, rs.comment_off, hc ? comment : std::string());
        rs.has_comment.push_back(hc);
    }
}

}  // namespace sa
