// Host-side inputs: reference contigs (2-bit PackedSeq form) and read batches.
// FASTA: src/io/fasta.rs:116-165; FASTQ: src/io/fastq.rs:19-100; headers split
// as src/io/mod.rs:33-40; wildcard bases encoded as src/packed_seq.rs:50-92; gzip
// inputs as src/io/xopen.rs:9-20.
#include "host_input.h"

#include <dlfcn.h>
#include <fcntl.h>
#include <unistd.h>

#include <cerrno>
#include <cmath>
#include <cstring>
#include <mutex>

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

struct ByteSource::Gz {
    ZStream zs{};
    std::vector<unsigned char> in;
    bool input_end = false, member_done = false, any_input = false, open = false;
    ~Gz() {
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

size_t LineReader::read_line(std::string& out) {
    size_t total = 0;
    for (;;) {
        if (pos_ >= end_ && !fill()) return total;
        const char* b = buf_.data() + pos_;
        const size_t avail = end_ - pos_;
        const char* nl = static_cast<const char*>(std::memchr(b, '\n', avail));
        const size_t take = nl ? (size_t)(nl - b) + 1 : avail;
        out.append(b, take);
        pos_ += take;
        total += take;
        if (nl) return total;
    }
}

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
    LineReader f(path);
    std::string line;
    bool have = false;
    Contig cur;
    for (;;) {
        line.clear();
        if (!f.read_line(line)) break;
        if (line[0] == '>') {
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
    if (fasta_) have_header_ = in_.read_line(header_) > 0;
}

// Vec::pop of the line end, then a '\r' (src/io/fastq.rs:62-66)
static void drop_line_end(std::string& s) {
    if (!s.empty()) s.pop_back();
    if (!s.empty() && s.back() == '\r') s.pop_back();
}

size_t ReadParser::parse(ReadStore& rs, size_t max_records) {
    size_t n = 0;
    if (fasta_) {
        rs.has_qual = false;
        while (n < max_records && have_header_) {
            bool hc = false;
            split_header(header_.substr(1), name_, comment_, hc);
            seq_.clear();
            have_header_ = false;
            for (;;) {
                line_.clear();
                if (!in_.read_line(line_)) break;
                if (line_[0] == '>') {
                    header_.swap(line_);
                    have_header_ = true;
                    break;
                }
                std::string t = trim_end(line_);
                for (char& c : t) c = (char)toupper((unsigned char)c);
                seq_ += t;
            }
            push_str(rs.seq, rs.seq_off, seq_);
            push_str(rs.names, rs.name_off, name_);
            push_str(rs.comments, rs.comment_off, hc ? comment_ : std::string());
            rs.has_comment.push_back(hc);
            n++;
        }
        return n;
    }
    rs.has_qual = true;
    rs.qual_off_unused = 0;
    while (n < max_records) {
        line_.clear();
        if (!in_.read_line(line_)) break;
        if (line_[0] != '@') throw Error(SA_ERR_FORMAT, "FASTQ record must start with '@'");
        bool hc = false;
        split_header(line_.substr(1), name_, comment_, hc);
        if (name_.empty()) throw Error(SA_ERR_FORMAT, "Record identifier is empty");
        if (name_.size() >= 2 &&
            (name_.compare(name_.size() - 2, 2, "/1") == 0 || name_.compare(name_.size() - 2, 2, "/2") == 0))
            name_.resize(name_.size() - 2);
        seq_.clear();
        in_.read_line(seq_);
        drop_line_end(seq_);
        line_.clear();
        in_.read_line(line_);
        qual_.clear();
        in_.read_line(qual_);
        drop_line_end(qual_);
        if (seq_.size() != qual_.size())
            throw Error(SA_ERR_FORMAT, "Found " + std::to_string(seq_.size()) + " nucleotides but " +
                                           std::to_string(qual_.size()) + " quality values in record '" + name_ + "'");
        for (char& c : seq_) c = (char)toupper((unsigned char)c);
        push_str(rs.seq, rs.seq_off, seq_);
        rs.qual += qual_;
        push_str(rs.names, rs.name_off, name_);
        push_str(rs.comments, rs.comment_off, hc ? comment_ : std::string());
        rs.has_comment.push_back(hc);
        n++;
    }
    return n;
}

void load_reads(const std::string& path, ReadStore& rs) {
    ReadParser p(path);
    reset_read_store(rs, !p.fasta());
    p.parse(rs, SIZE_MAX);
}

}  // namespace sa
