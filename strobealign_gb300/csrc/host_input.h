// Input files: plain or gzip bytes, buffered lines, and an incremental FASTQ / FASTA
// read parser, so that inputs can be read in batches while earlier batches map.
#pragma once
#include "host_state.h"

#include <atomic>
#include <memory>
#include <string>
#include <string_view>
#include <vector>

namespace sa {

// The bytes of an input: "-" is standard input; a name ending in ".gz" is gzip, every
// member decoded in turn (src/io/xopen.rs:9-20 opens a MultiGzDecoder by the same
// rule).  zlib is loaded at run time (libz.so.1) when the first .gz input is opened.
class ByteSource {
  public:
    explicit ByteSource(const std::string& path);
    ~ByteSource();
    ByteSource(const ByteSource&) = delete;
    ByteSource& operator=(const ByteSource&) = delete;
    // up to n bytes into dst; 0 at the end of the input
    size_t read(char* dst, size_t n);
    uint64_t file_bytes() const { return raw_; }  // bytes taken from the file so far
    bool gzip() const { return gz_ != nullptr; }

  private:
    size_t read_file(char* dst, size_t n);
    size_t inflate_some(char* dst, size_t n);  // gzip: the next decoded bytes, 0 at the end
    std::string path_;
    int fd_ = -1;
    bool own_fd_ = false;
    std::atomic<uint64_t> raw_{0};
    struct Gz;
    std::unique_ptr<Gz> gz_;
};

// Buffered lines of a ByteSource (BufRead::read_until on b'\n')
class LineReader {
  public:
    explicit LineReader(const std::string& path);
    // the next line without its '\n' as a view that stays valid until the next call;
    // newline tells whether the line ended with '\n' (not at the end of the input);
    // false at the end of the input
    bool next(std::string_view& line, bool& newline);
    int peek();  // the next byte, -1 at the end
    const ByteSource& source() const { return src_; }

  private:
    bool fill();
    ByteSource src_;
    std::vector<char> buf_;
    size_t pos_ = 0, end_ = 0;
    bool eof_ = false;
    std::string spill_;  // a line that crosses the end of the buffer
};

// Incremental read parser: FASTA when the first byte is '>' (src/io/reads.rs:121-132),
// else FASTQ records as src/io/fastq.rs:22-94 reads them (names split at the first
// blank, a trailing /1 or /2 dropped, sequences upper-cased, the last byte of the
// sequence and quality lines dropped as the line end and a '\r' before it).
class ReadParser {
  public:
    explicit ReadParser(const std::string& path);
    // appends up to max_records records to rs; returns how many, 0 at the end of the input
    size_t parse(ReadStore& rs, size_t max_records);
    bool fasta() const { return fasta_; }
    uint64_t file_bytes() const { return in_.source().file_bytes(); }

  private:
    LineReader in_;
    bool fasta_ = false;
    std::string header_;  // FASTA: the next record's header line, read ahead
    bool have_header_ = false;
};

// Records of reads in file order as InterleavedIterator forms them (src/io/reads.rs:
// 68-113): a read and the next one are a pair when their names are equal, any other read
// is single-end.  rec_read gets each record's first read and then the number of reads the
// records cover (records + 1 entries).  Unless at_end, a last read without a successor
// is left out: the next read of the input may be its mate.
void pair_records_by_name(const sa_read_batch& reads, bool at_end, std::vector<uint32_t>& rec_read);

// An empty store (offset arrays holding their leading 0)
void reset_read_store(ReadStore& rs, bool has_qual);
inline size_t read_store_size(const ReadStore& rs) { return rs.seq_off.empty() ? 0 : rs.seq_off.size() - 1; }
// Moves records [from, n) of rs into tail (reset first); rs keeps [0, from)
void split_read_store(ReadStore& rs, size_t from, ReadStore& tail);

}  // namespace sa
