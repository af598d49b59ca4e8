// Host-side inputs: reference contigs (2-bit PackedSeq form) and read batches.
// FASTA: src/io/fasta.rs:116-165; FASTQ: src/io/fastq.rs:19-100; headers split
// as src/io/mod.rs:33-40; wildcard bases encoded as src/packed_seq.rs:50-92; gzip
// inputs as src/io/xopen.rs:9-20.
#include "host_input.h"

#include <dlfcn.h>
#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <exception>
#include <mutex>
#include <thread>

namespace sa {

// ---------------------------------------------------------------- gzip through zlib
// zlib's z_stream as its public header lays it out (identical on LP64 x86-64 and
// aarch64); the library is opened by name, so no zlib header is needed to build.
struct ZStream {
    const unsigned char* next_in;
    unsigned avail_in;
    unsigned long total_in;
    unsigned char* next_out;
    unsigned avail_out;
    unsigned long total_out;
    const char* msg;
    void* state;
    void* zalloc;
    void* zfree;
    void* opaque;
    int data_type;
    unsigned long adler;
    unsigned long reserved;
};

namespace {
constexpr int Z_OK_ = 0, Z_STREAM_END_ = 1, Z_BUF_ERROR_ = -5, Z_NO_FLUSH_ = 0;

struct Zlib {
    int (*inflate_init2)(ZStream*, int, const char*, int) = nullptr;
    int (*inflate)(ZStream*, int) = nullptr;
    int (*inflate_end)(ZStream*) = nullptr;
    int (*inflate_reset)(ZStream*) = nullptr;
    const char* (*version)() = nullptr;
    std::string error;
};

const Zlib& zlib() {
    static Zlib z;
    static std::once_flag once;
    std::call_once(once, [] {
        void* h = dlopen("libz.so.1", RTLD_NOW | RTLD_LOCAL);
        if (!h) h = dlopen("libz.so", RTLD_NOW | RTLD_LOCAL);
        if (!h) {
            z.error = "gzip input needs zlib (libz.so.1), which could not be loaded";
            return;
        }
        z.inflate_init2 = (int (*)(ZStream*, int, const char*, int))dlsym(h, "inflateInit2_");
        z.inflate = (int (*)(ZStream*, int))dlsym(h, "inflate");
        z.inflate_end = (int (*)(ZStream*))dlsym(h, "inflateEnd");
        z.inflate_reset = (int (*)(ZStream*))dlsym(h, "inflateReset");
        z.version = (const char* (*)())dlsym(h, "zlibVersion");
        if (!z.inflate_init2 || !z.inflate || !z.inflate_end || !z.inflate_reset || !z.version)
            z.error = "libz.so.1 lacks the inflate entry points";
    });
    return z;
}

bool ends_with(const std::string& s, const char* suffix) {
    const size_t n = std::strlen(suffix);
    return s.size() >= n && s.compare(s.size() - n, n, suffix) == 0;
}
}  // namespace

// gzip decoding runs on a thread of its own, a few blocks ahead of the reader, so that
// inflating and parsing overlap
struct ByteSource::Gz {
    ZStream zs{};
    std::vector<unsigned char> in;
    bool input_end = false, member_done = false, any_input = false, open = false;
    // decoded blocks handed to read(): at most kAhead queued
    static constexpr size_t kBlock = (size_t)4 << 20, kAhead = 4;
    std::thread worker;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<std::vector<char>> ready, spare;
    bool done = false, stop = false;
    std::exception_ptr err;
    std::vector<char> cur;  // the block read() is taking bytes from
    size_t cur_pos = 0;
    ~Gz() {
        if (worker.joinable()) {
            {
                std::lock_guard<std::mutex> g(mu);
                stop = true;
            }
            cv.notify_all();
            worker.join();
        }
        if (open) zlib().inflate_end(&zs);
    }
};

ByteSource::ByteSource(const std::string& path) : path_(path) {
    if (path == "-") {
        fd_ = 0;
    } else {
        fd_ = ::open(path.c_str(), O_RDONLY | O_CLOEXEC);
        if (fd_ < 0) throw Error(SA_ERR_IO, "cannot open " + path + ": " + std::strerror(errno));
        own_fd_ = true;
    }
    if (path != "-" && ends_with(path, ".gz")) {
        const Zlib& z = zlib();
        if (!z.error.empty()) {
            ::close(fd_);
            throw Error(SA_ERR_IO, path + ": " + z.error);
        }
        gz_ = std::make_unique<Gz>();
        gz_->in.resize((size_t)1 << 20);
        // window bits 15 + 16: gzip members only
        if (z.inflate_init2(&gz_->zs, 15 + 16, z.version(), (int)sizeof(ZStream)) != Z_OK_) {
            ::close(fd_);
            throw Error(SA_ERR_IO, path + ": zlib inflateInit2 failed");
        }
        gz_->open = true;
    }
}

ByteSource::~ByteSource() {
    gz_.reset();
    if (own_fd_ && fd_ >= 0) ::close(fd_);
}

size_t ByteSource::read_file(char* dst, size_t n) {
    for (;;) {
        const ssize_t k = ::read(fd_, dst, n);
        if (k >= 0) {
            raw_ += (uint64_t)k;
            return (size_t)k;
        }
        if (errno != EINTR) throw Error(SA_ERR_IO, "read error on " + path_ + ": " + std::strerror(errno));
    }
}

size_t ByteSource::read(char* dst, size_t n) {
    if (!gz_) return read_file(dst, n);
    Gz& g = *gz_;
    if (!g.worker.joinable() && !g.done) {
        g.worker = std::thread([this] {
            Gz& w = *gz_;
            try {
                for (;;) {
                    std::vector<char> blk;
                    {
                        std::unique_lock<std::mutex> l(w.mu);
                        w.cv.wait(l, [&] { return w.stop || w.ready.size() < Gz::kAhead; });
                        if (w.stop) return;
                        if (!w.spare.empty()) {
                            blk.swap(w.spare.front());
                            w.spare.pop_front();
                        }
                    }
                    blk.resize(Gz::kBlock);
                    size_t got = 0;
                    while (got < blk.size()) {
                        const size_t k = inflate_some(blk.data() + got, blk.size() - got);
                        if (k == 0) break;
                        got += k;
                    }
                    blk.resize(got);
                    std::lock_guard<std::mutex> l(w.mu);
                    if (got) w.ready.push_back(std::move(blk));
                    if (got < Gz::kBlock) {
                        w.done = true;
                        w.cv.notify_all();
                        return;
                    }
                    w.cv.notify_all();
                }
            } catch (...) {
                std::lock_guard<std::mutex> l(w.mu);
                w.err = std::current_exception();
                w.done = true;
                w.cv.notify_all();
            }
        });
    }
    size_t out = 0;
    while (out < n) {
        if (g.cur_pos >= g.cur.size()) {
            std::unique_lock<std::mutex> l(g.mu);
            if (!g.cur.empty()) {
                g.cur.clear();
                g.spare.push_back(std::move(g.cur));
                g.cur = std::vector<char>();
            }
            g.cur_pos = 0;
            g.cv.wait(l, [&] { return !g.ready.empty() || g.done; });
            if (g.ready.empty()) {
                if (g.err) std::rethrow_exception(g.err);
                break;  // the end of the input
            }
            g.cur.swap(g.ready.front());
            g.ready.pop_front();
            g.cv.notify_all();
        }
        const size_t take = std::min(n - out, g.cur.size() - g.cur_pos);
        std::memcpy(dst + out, g.cur.data() + g.cur_pos, take);
        g.cur_pos += take;
        out += take;
        if (out) break;  // hand back what is there
    }
    return out;
}

size_t ByteSource::inflate_some(char* dst, size_t n) {
    Gz& g = *gz_;
    const Zlib& z = zlib();
    if (n > ((size_t)1 << 30)) n = (size_t)1 << 30;
    for (;;) {
        if (g.zs.avail_in == 0 && !g.input_end) {
            const size_t k = read_file(reinterpret_cast<char*>(g.in.data()), g.in.size());
            if (k == 0) g.input_end = true;
            else g.any_input = true;
            g.zs.next_in = g.in.data();
            g.zs.avail_in = (unsigned)k;
        }
        if (g.member_done) {
            // the next member starts right after this one; the input ends after a member
            if (g.zs.avail_in == 0) return 0;
            z.inflate_reset(&g.zs);
            g.member_done = false;
        }
        if (!g.any_input) return 0;  // an empty file holds no records
        g.zs.next_out = reinterpret_cast<unsigned char*>(dst);
        g.zs.avail_out = (unsigned)n;
        const int rc = z.inflate(&g.zs, Z_NO_FLUSH_);
        const size_t produced = n - g.zs.avail_out;
        if (rc == Z_STREAM_END_) {
            g.member_done = true;
        } else if (rc == Z_BUF_ERROR_) {
            if (g.input_end && g.zs.avail_in == 0 && produced == 0)
                throw Error(SA_ERR_FORMAT, path_ + ": unexpected end of gzip data");
        } else if (rc != Z_OK_) {
            throw Error(SA_ERR_FORMAT, path_ + ": invalid gzip data" + (g.zs.msg ? std::string(" (") + g.zs.msg + ")" : ""));
        } else if (produced == 0 && g.input_end && g.zs.avail_in == 0) {
            throw Error(SA_ERR_FORMAT, path_ + ": unexpected end of gzip data");
        }
        if (produced) return produced;
    }
}

// ---------------------------------------------------------------- lines
LineReader::LineReader(const std::string& path) : src_(path), buf_((size_t)4 << 20) {}

bool LineReader::fill() {
    if (eof_) return false;
    if (pos_ < end_) return true;
    pos_ = 0;
    end_ = src_.read(buf_.data(), buf_.size());
    if (end_ == 0) eof_ = true;
    return end_ > 0;
}

int LineReader::peek() {
    if (pos_ >= end_ && !fill()) return -1;
    return (unsigned char)buf_[pos_];
}

bool LineReader::next(std::string_view& line, bool& newline) {
    if (pos_ >= end_ && !fill()) return false;
    const char* b = buf_.data() + pos_;
    const char* nl = static_cast<const char*>(std::memchr(b, '\n', end_ - pos_));
    if (nl) {
        line = std::string_view(b, (size_t)(nl - b));
        pos_ += line.size() + 1;
        newline = true;
        return true;
    }
    // the line runs past the buffer: gather it
    spill_.assign(b, end_ - pos_);
    pos_ = end_;
    newline = false;
    while (fill()) {
        const char* c = buf_.data() + pos_;
        const char* n2 = static_cast<const char*>(std::memchr(c, '\n', end_ - pos_));
        const size_t take = n2 ? (size_t)(n2 - c) : end_ - pos_;
        spill_.append(c, take);
        pos_ += take;
        if (n2) {
            pos_++;
            newline = true;
            break;
        }
    }
    line = spill_;
    return true;
}

// Lines the reference reads into a String (read_line) must be UTF-8, or the read fails
// with an I/O error: every line of a FASTA file, and a FASTQ record's header lines.
// RFC 3629 well-formedness (no overlong forms, no surrogates, nothing above U+10FFFF).
static bool utf8_ok(std::string_view s) {
    const auto* p = reinterpret_cast<const unsigned char*>(s.data());
    const size_t n = s.size();
    size_t i = 0;
    while (i < n) {
        // ASCII runs, eight bytes at a time
        while (i + 8 <= n) {
            uint64_t w;
            std::memcpy(&w, p + i, 8);
            if (w & 0x8080808080808080ULL) break;
            i += 8;
        }
        if (i >= n) break;
        const unsigned c = p[i];
        if (c < 0x80) {
            i++;
            continue;
        }
        size_t len;
        unsigned lo = 0x80, hi = 0xBF;  // range of the second byte
        if (c >= 0xC2 && c <= 0xDF) len = 2;
        else if (c == 0xE0) len = 3, lo = 0xA0;
        else if (c >= 0xE1 && c <= 0xEC) len = 3;
        else if (c == 0xED) len = 3, hi = 0x9F;
        else if (c >= 0xEE && c <= 0xEF) len = 3;
        else if (c == 0xF0) len = 4, lo = 0x90;
        else if (c >= 0xF1 && c <= 0xF3) len = 4;
        else if (c == 0xF4) len = 4, hi = 0x8F;
        else return false;
        if (i + len > n) return false;
        if (p[i + 1] < lo || p[i + 1] > hi) return false;
        for (size_t k = 2; k < len; k++)
            if (p[i + k] < 0x80 || p[i + k] > 0xBF) return false;
        i += len;
    }
    return true;
}

static void require_utf8(std::string_view line) {
    if (!utf8_ok(line)) throw Error(SA_ERR_FORMAT, "stream did not contain valid UTF-8");
}

// trim_ascii_end: space, tab, line feed, form feed and carriage return (not vertical tab)
static std::string_view trim_end_view(std::string_view s) {
    size_t e = s.size();
    while (e > 0 && (s[e - 1] == ' ' || s[e - 1] == '\t' || s[e - 1] == '\n' || s[e - 1] == '\r' ||
                     s[e - 1] == '\f'))
        e--;
    return s.substr(0, e);
}

// split_header on a view: name up to the first blank, the comment after it
static void split_header_view(std::string_view h, std::string_view& name, std::string_view& comment,
                              bool& has_comment) {
    const std::string_view t = trim_end_view(h);
    const size_t p = t.find_first_of(" \t");
    if (p == std::string_view::npos) {
        name = t;
        comment = std::string_view();
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
    LineReader f(path);
    std::string_view line;
    bool nl = false, have = false;
    Contig cur;
    while (f.next(line, nl)) {
        require_utf8(line);
        if (!line.empty() && line[0] == '>') {
            if (have) out.push_back(std::move(cur));
            cur = Contig();
            std::string_view name, c;
            bool hc;
            split_header_view(line.substr(1), name, c, hc);
            cur.name.assign(name);
            have = true;
        } else if (have) {
            for (char ch : trim_end_view(line)) cur.push((uint8_t)ch);
        } else if (!trim_end_view(line).empty()) {
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

void pair_records_by_name(const sa_read_batch& reads, bool at_end, std::vector<uint32_t>& rec_read) {
    const size_t n = reads.n;
    if (n >= UINT32_MAX) throw Error(SA_ERR_INVALID, "batch too large");
    rec_read.clear();
    rec_read.reserve(n + 1);
    auto name = [&](size_t i) {
        return std::string_view(reads.names + reads.name_offsets[i], reads.name_offsets[i + 1] - reads.name_offsets[i]);
    };
    size_t i = 0;
    while (i < n) {
        if (i + 1 == n && !at_end) break;
        rec_read.push_back((uint32_t)i);
        i += i + 1 < n && name(i) == name(i + 1) ? 2 : 1;
    }
    rec_read.push_back((uint32_t)i);
}

void reset_read_store(ReadStore& rs, bool has_qual) {
    rs = ReadStore();
    rs.seq_off.push_back(0);
    rs.name_off.push_back(0);
    rs.comment_off.push_back(0);
    rs.has_qual = has_qual;
}

void split_read_store(ReadStore& rs, size_t from, ReadStore& tail) {
    const size_t n = read_store_size(rs);
    reset_read_store(tail, rs.has_qual);
    if (from >= n) return;
    const uint64_t s0 = rs.seq_off[from], n0 = rs.name_off[from], c0 = rs.comment_off[from];
    tail.seq.assign(rs.seq, s0, std::string::npos);
    if (rs.has_qual) tail.qual.assign(rs.qual, s0, std::string::npos);
    tail.names.assign(rs.names, n0, std::string::npos);
    tail.comments.assign(rs.comments, c0, std::string::npos);
    for (size_t i = from + 1; i <= n; i++) {
        tail.seq_off.push_back(rs.seq_off[i] - s0);
        tail.name_off.push_back(rs.name_off[i] - n0);
        tail.comment_off.push_back(rs.comment_off[i] - c0);
    }
    tail.has_comment.assign(rs.has_comment.begin() + (ptrdiff_t)from, rs.has_comment.end());
    rs.seq.resize(s0);
    if (rs.has_qual) rs.qual.resize(s0);
    rs.names.resize(n0);
    rs.comments.resize(c0);
    rs.seq_off.resize(from + 1);
    rs.name_off.resize(from + 1);
    rs.comment_off.resize(from + 1);
    rs.has_comment.resize(from);
}

ReadParser::ReadParser(const std::string& path) : in_(path) {
    fasta_ = in_.peek() == '>';
    if (fasta_) {
        std::string_view h;
        bool nl;
        have_header_ = in_.next(h, nl);
        if (have_header_) {
            require_utf8(h);
            header_.assign(h);
        }
    }
}

namespace {
// appends s with a-z upper-cased (u8::to_ascii_uppercase); a branch-free byte loop the
// compiler vectorizes
void append_upper(std::string& out, std::string_view s) {
    const size_t o = out.size();
    out.append(s);
    unsigned char* p = reinterpret_cast<unsigned char*>(&out[o]);
    for (size_t i = 0; i < s.size(); i++) {
        const unsigned char c = p[i];
        p[i] = (unsigned char)(c - (((unsigned char)(c - 'a') < 26) << 5));
    }
}

// the sequence / quality line as read_until and Vec::pop leave it (src/io/fastq.rs:61-76):
// the last byte goes (the '\n', or a real byte at the end of the input), then a '\r'
std::string_view fastq_line(std::string_view l, bool newline) {
    if (!newline && !l.empty()) l.remove_suffix(1);
    if (!l.empty() && l.back() == '\r') l.remove_suffix(1);
    return l;
}
}  // namespace

size_t ReadParser::parse(ReadStore& rs, size_t max_records) {
    size_t n = 0;
    std::string_view line, name, comment;
    bool nl = false, hc = false;
    if (fasta_) {
        rs.has_qual = false;
        while (n < max_records && have_header_) {
            split_header_view(std::string_view(header_).substr(1), name, comment, hc);
            rs.names.append(name);
            rs.name_off.push_back(rs.names.size());
            rs.comments.append(hc ? comment : std::string_view());
            rs.comment_off.push_back(rs.comments.size());
            rs.has_comment.push_back(hc);
            have_header_ = false;
            while (in_.next(line, nl)) {
                require_utf8(line);
                if (!line.empty() && line[0] == '>') {
                    header_.assign(line);
                    have_header_ = true;
                    break;
                }
                append_upper(rs.seq, trim_end_view(line));
            }
            rs.seq_off.push_back(rs.seq.size());
            n++;
        }
        return n;
    }
    rs.has_qual = true;
    rs.qual_off_unused = 0;
    while (n < max_records) {
        if (!in_.next(line, nl)) break;
        require_utf8(line);
        if (line.empty() || line[0] != '@') throw Error(SA_ERR_FORMAT, "FASTQ record must start with '@'");
        split_header_view(line.substr(1), name, comment, hc);
        if (name.empty()) throw Error(SA_ERR_FORMAT, "Record identifier is empty");
        if (name.size() >= 2 && name[name.size() - 2] == '/' && (name.back() == '1' || name.back() == '2'))
            name.remove_suffix(2);
        // the views die with the next line: keep the name now
        const size_t name0 = rs.names.size(), comment0 = rs.comments.size();
        rs.names.append(name);
        rs.comments.append(hc ? comment : std::string_view());
        std::string_view seq;
        if (in_.next(line, nl)) seq = fastq_line(line, nl);
        else seq = std::string_view();
        const size_t seq0 = rs.seq.size();
        append_upper(rs.seq, seq);
        const size_t L = rs.seq.size() - seq0;
        std::string_view plus;
        bool nl2;
        if (in_.next(plus, nl2)) require_utf8(plus);
        std::string_view qual;
        if (in_.next(line, nl)) qual = fastq_line(line, nl);
        else qual = std::string_view();
        if (L != qual.size()) {
            const std::string nm = rs.names.substr(name0);
            rs.names.resize(name0);
            rs.comments.resize(comment0);
            rs.seq.resize(seq0);
            throw Error(SA_ERR_FORMAT, "Found " + std::to_string(L) + " nucleotides but " +
                                           std::to_string(qual.size()) + " quality values in record '" + nm + "'");
        }
        rs.qual.append(qual);
        rs.seq_off.push_back(rs.seq.size());
        rs.name_off.push_back(rs.names.size());
        rs.comment_off.push_back(rs.comments.size());
        rs.has_comment.push_back(hc);
        n++;
    }
    return n;
}

void load_reads(const std::string& path, ReadStore& rs) {
    ReadParser p(path);
    reset_read_store(rs, !p.fasta());
    // room for a plain file's records up front (about half of a FASTQ is bases), so the
    // stores grow without copying
    struct stat st {};
    if (path != "-" && !ends_with(path, ".gz") && ::stat(path.c_str(), &st) == 0 && st.st_size > 0) {
        const size_t sz = (size_t)st.st_size;
        rs.seq.reserve(sz / 2 + 1024);
        if (!p.fasta()) rs.qual.reserve(sz / 2 + 1024);
        rs.names.reserve(sz / 16 + 1024);
        const size_t recs = sz / 64 + 16;
        rs.seq_off.reserve(recs);
        rs.name_off.reserve(recs);
        rs.comment_off.reserve(recs);
        rs.has_comment.reserve(recs);
    }
    p.parse(rs, SIZE_MAX);
}

}  // namespace sa
