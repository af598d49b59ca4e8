// Oracle (test infrastructure only): FASTA/FASTQ parsing and the SAM header.
// Restates src/io/{fasta,fastq,mod,sam}.rs.
#include "oracle.hpp"

#include <cstdio>
#include <fstream>
#include <sstream>
#include <algorithm>

namespace oracle {

// trim_ascii_end: space, tab, line feed, form feed and carriage return (not vertical tab)
static std::string trim_end(const std::string& s) {
    size_t e = s.size();
    while (e > 0 && (s[e - 1] == ' ' || s[e - 1] == '\t' || s[e - 1] == '\n' || s[e - 1] == '\r' ||
                     s[e - 1] == '\f'))
        e--;
    return s.substr(0, e);
}

// src/io/mod.rs:33-40
static void split_header(const std::string& h, std::string& name, std::string& comment, bool& has_comment) {
    std::string t = trim_end(h);
    size_t p = t.find_first_of(" \t");
    if (p == std::string::npos) {
        name = t;
        has_comment = false;
        comment.clear();
    } else {
        name = t.substr(0, p);
        comment = t.substr(p + 1);
        has_comment = true;
    }
}

// src/io/fasta.rs:116-165 (read_fasta)
bool read_fasta(const std::string& path, std::vector<RefSeq>& out, std::string& err) {
    std::ifstream f(path, std::ios::binary);
    if (!f) { err = "cannot open " + path; return false; }
    std::string line;
    bool have = false;
    RefSeq cur;
    while (std::getline(f, line)) {
        if (!line.empty() && line[0] == '>') {
            if (have) out.push_back(std::move(cur));
            cur = RefSeq();
            std::string c;
            bool hc;
            split_header(line.substr(1), cur.name, c, hc);
            have = true;
        } else if (have) {
            std::string t = trim_end(line);
            for (char ch : t) cur.seq.push((uint8_t)ch);
        } else if (!trim_end(line).empty()) {
            err = "FASTA file must start with '>'";
            return false;
        }
    }
    if (have) out.push_back(std::move(cur));
    return true;
}

// src/io/fastq.rs:19-100 and src/io/fasta.rs:63-110 (FastaReader used for reads)
bool read_fastq_file(const std::string& path, std::vector<SequenceRecord>& out, std::string& err) {
    std::ifstream f(path, std::ios::binary);
    if (!f) { err = "cannot open " + path; return false; }
    int first = f.peek();
    if (first == '>') {
        std::string line;
        SequenceRecord cur;
        bool have = false;
        while (std::getline(f, line)) {
            if (!line.empty() && line[0] == '>') {
                if (have) out.push_back(cur);
                cur = SequenceRecord();
                split_header(line.substr(1), cur.name, cur.comment, cur.has_comment);
                have = true;
            } else {
                std::string t = trim_end(line);
                for (char& c : t) c = (char)toupper((unsigned char)c);
                cur.seq += t;
            }
        }
        if (have) out.push_back(cur);
        return true;
    }
    std::string l1, l2, l3, l4;
    while (std::getline(f, l1)) {
        if (l1.empty() || l1[0] != '@') { err = "Record must start with '@'"; return false; }
        SequenceRecord r;
        split_header(l1.substr(1), r.name, r.comment, r.has_comment);
        if (r.name.empty()) { err = "Record identifier is empty"; return false; }
        if (r.name.size() >= 2 && r.name.compare(r.name.size() - 2, 2, "/1") == 0) { r.name.resize(r.name.size() - 2); r.end = 1; }
        else if (r.name.size() >= 2 && r.name.compare(r.name.size() - 2, 2, "/2") == 0) { r.name.resize(r.name.size() - 2); r.end = 2; }
        std::getline(f, l2);
        std::getline(f, l3);
        std::getline(f, l4);
        if (!l2.empty() && l2.back() == '\r') l2.pop_back();
        if (!l4.empty() && l4.back() == '\r') l4.pop_back();
        for (char& c : l2) c = (char)toupper((unsigned char)c);
        if (l2.size() != l4.size()) { err = "sequence/quality length mismatch in " + r.name; return false; }
        r.seq = l2;
        r.qual = l4;
        r.has_qual = true;
        out.push_back(std::move(r));
    }
    return true;
}

// src/io/sam.rs:176-200
std::string sam_header(const std::vector<RefSeq>& refs, const std::string* cmd_line, const std::string& version,
                       const std::string* rg_id, const std::vector<std::string>& rg_fields) {
    std::string h = "@HD\tVN:1.6\tSO:unsorted\n";
    for (auto& r : refs) h += "@SQ\tSN:" + r.name + "\tLN:" + std::to_string(r.seq.len) + "\n";
    if (rg_id) {
        h += "@RG\tID:" + *rg_id;
        for (auto& f : rg_fields) h += "\t" + f;
        h += "\n";
    }
    if (cmd_line) h += "@PG\tID:strobealign\tPN:strobealign\tVN:" + version + "\tCL:" + *cmd_line + "\n";
    return h;
}

}  // namespace oracle
