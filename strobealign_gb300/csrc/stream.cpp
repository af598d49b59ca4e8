// File-to-file mapping: a reader thread parses (and gunzips) the input into batches of
// whole chunks, the calling thread maps each batch on the device, and a writer thread
// writes the outputs in input order, so parsing batch k+1 and writing batch k-1 overlap
// mapping batch k.  This is the shape of the reference's CLI loop (src/main.rs:555-604
// reads records into chunks on a reader thread; :653-667 writes them in chunk order),
// with a batch of many chunks as the unit handed to the GPU.
#include "stream.h"

#include <algorithm>
#include <atomic>
#include <cerrno>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <exception>
#include <mutex>
#include <thread>

#include "host_input.h"

namespace sa {

namespace {

struct InBatch {
    ReadStore r1, r2;
    size_t records = 0;  // interleaved input: records (single-end or pairs) of r1's reads
};

template <class T>
class BoundedQueue {
  public:
    explicit BoundedQueue(size_t cap) : cap_(cap ? cap : 1) {}
    // false when the queue was closed for pushing
    bool push(T&& v) {
        std::unique_lock<std::mutex> g(mu_);
        not_full_.wait(g, [&] { return q_.size() < cap_ || closed_; });
        if (closed_) return false;
        q_.push_back(std::move(v));
        not_empty_.notify_one();
        return true;
    }
    // false at the end (closed and drained)
    bool pop(T& v) {
        std::unique_lock<std::mutex> g(mu_);
        not_empty_.wait(g, [&] { return !q_.empty() || closed_; });
        if (q_.empty()) return false;
        v = std::move(q_.front());
        q_.pop_front();
        not_full_.notify_one();
        return true;
    }
    void close() {
        std::lock_guard<std::mutex> g(mu_);
        closed_ = true;
        not_empty_.notify_all();
        not_full_.notify_all();
    }

  private:
    std::mutex mu_;
    std::condition_variable not_full_, not_empty_;
    std::deque<T> q_;
    size_t cap_;
    bool closed_ = false;
};

sa_read_batch view_of(const ReadStore& s) {
    sa_read_batch v{};
    v.n = read_store_size(s);
    v.seq = s.seq.data();
    v.seq_offsets = s.seq_off.data();
    v.qual = s.has_qual ? s.qual.data() : nullptr;
    v.names = s.names.data();
    v.name_offsets = s.name_off.data();
    v.comments = s.comments.data();
    v.comment_offsets = s.comment_off.data();
    return v;
}

double since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

// Records of the pending stores [0, cut) that form whole chunks: records go into a
// chunk until its nucleotides (both mates) exceed chunk_size (src/main.rs:591-604); the
// last chunk counts as whole only at the end of the input.
size_t whole_chunks(const ReadStore& a, const ReadStore* b, uint64_t chunk_size, bool at_end) {
    const size_t n = read_store_size(a);
    auto off = [&](size_t j) { return a.seq_off[j] + (b ? b->seq_off[j] : 0); };
    size_t cut = 0;
    for (size_t i = 0; i < n;) {
        size_t j = i;
        const uint64_t base = off(i);
        bool full = false;
        while (j < n) {
            j++;
            if (off(j) - base > chunk_size) {
                full = true;
                break;
            }
        }
        if (!full && !at_end) break;
        cut = j;
        i = j;
    }
    return cut;
}

// Interleaved input: as whole_chunks over the records pair_records_by_name forms from the
// pending reads; returns the cut in reads and sets records to the records before it.
size_t whole_chunks_interleaved(const ReadStore& a, uint64_t chunk_size, bool at_end, std::vector<uint32_t>& rec_read,
                                size_t& records) {
    const sa_read_batch v = view_of(a);
    pair_records_by_name(v, at_end, rec_read);
    const size_t n = rec_read.size() - 1;
    auto off = [&](size_t j) { return a.seq_off[rec_read[j]]; };
    size_t cut = 0;
    for (size_t i = 0; i < n;) {
        size_t j = i;
        const uint64_t base = off(i);
        bool full = false;
        while (j < n) {
            j++;
            if (off(j) - base > chunk_size) {
                full = true;
                break;
            }
        }
        if (!full && !at_end) break;
        cut = j;
        i = j;
    }
    records = cut;
    return rec_read[cut];
}

}  // namespace

StreamResult map_files(Mapper& m, const std::string& reads1, const std::string* reads2, const std::string& out_path,
                       const StreamConfig& cfg) {
    const auto t0 = std::chrono::steady_clock::now();
    const uint64_t batch_bases = cfg.batch_bases ? cfg.batch_bases : ((uint64_t)1 << 29);
    const uint64_t chunk_size = m.mapping_params().chunk_size;
    // open everything before any thread starts, so that a bad path fails the call cleanly
    auto p1 = std::make_unique<ReadParser>(reads1);
    std::unique_ptr<ReadParser> p2;
    if (reads2) p2 = std::make_unique<ReadParser>(*reads2);
    std::FILE* out = nullptr;
    if (out_path == "-") {
        out = stdout;
    } else {
        out = std::fopen(out_path.c_str(), cfg.append ? "ab" : "wb");
        if (!out) throw Error(SA_ERR_IO, "cannot open " + out_path + " for writing: " + std::strerror(errno));
    }
    // a large buffer for a file this call opened (standard output keeps its own: a
    // buffer installed there would outlive this call)
    std::vector<char> obuf;
    if (out != stdout) {
        obuf.resize((size_t)8 << 20);
        std::setvbuf(out, obuf.data(), _IOFBF, obuf.size());
    }
    auto close_out = [&]() {
        if (out && out != stdout) std::fclose(out);
        else if (out) std::fflush(out);
        out = nullptr;
    };
    // closes the file on any early exit, before its buffer goes
    struct OutGuard {
        std::FILE*& f;
        ~OutGuard() {
            if (f && f != stdout) std::fclose(f);
            else if (f) std::fflush(f);
        }
    } guard{out};

    StreamResult res;
    BoundedQueue<std::unique_ptr<InBatch>> inq(cfg.read_ahead ? cfg.read_ahead : 2);
    BoundedQueue<sa_output> outq(2);
    std::exception_ptr reader_err, writer_err;
    std::atomic<uint64_t> bytes_out{0};

    std::thread reader([&] {
        try {
            auto pend = std::make_unique<InBatch>();
            reset_read_store(pend->r1, !p1->fasta());
            if (p2) reset_read_store(pend->r2, !p2->fasta());
            // room for a batch up front: the stores then grow without copying
            const uint64_t per_file = (p2 ? batch_bases / 2 : batch_bases) + (batch_bases >> 4);
            auto reserve = [&](ReadStore& rs, size_t records) {
                rs.seq.reserve(per_file);
                if (rs.has_qual) rs.qual.reserve(per_file);
                rs.seq_off.reserve(records + 1);
                rs.name_off.reserve(records + 1);
                rs.comment_off.reserve(records + 1);
                rs.has_comment.reserve(records);
                rs.names.reserve(records * 16);
            };
            size_t rec_est = (size_t)std::min<uint64_t>(per_file / 100 + 1024, (uint64_t)1 << 24);
            reserve(pend->r1, rec_est);
            if (p2) reserve(pend->r2, rec_est);
            bool at_end = false;
            std::vector<uint32_t> rec_read;
            while (true) {
                // parse until the pending records hold a batch's bases and one whole chunk
                size_t cut = 0, records = 0;
                for (;;) {
                    const uint64_t bases = pend->r1.seq.size() + (p2 ? pend->r2.seq.size() : 0);
                    if (at_end || bases >= batch_bases) {
                        if (cfg.interleaved) {
                            cut = whole_chunks_interleaved(pend->r1, chunk_size, at_end, rec_read, records);
                        } else {
                            cut = whole_chunks(pend->r1, p2 ? &pend->r2 : nullptr, chunk_size, at_end);
                            records = cut;
                        }
                        if (cut > 0 || at_end) break;
                    }
                    // records to parse next: about what the batch still lacks, at the
                    // mean record length so far (150 nt per mate before the first)
                    const size_t have = read_store_size(pend->r1);
                    const double per_rec = have ? (double)bases / (double)have : (p2 ? 300.0 : 150.0);
                    const double lack = bases < batch_bases ? (double)(batch_bases - bases) : (double)chunk_size;
                    const size_t step = (size_t)std::min(65536.0, std::max(256.0, lack / per_rec + 1.0));
                    size_t k1 = 0, k2 = 0;
                    if (p2) {
                        std::exception_ptr e2;
                        std::thread t2([&] {
                            try {
                                k2 = p2->parse(pend->r2, step);
                            } catch (...) {
                                e2 = std::current_exception();
                            }
                        });
                        try {
                            k1 = p1->parse(pend->r1, step);
                        } catch (...) {
                            t2.join();
                            throw;
                        }
                        t2.join();
                        if (e2) std::rethrow_exception(e2);
                        // pairs as zip forms them (src/io/reads.rs:56-62): they end with
                        // the shorter file
                        if (k1 != k2) {
                            ReadStore drop;
                            const size_t n = std::min(read_store_size(pend->r1), read_store_size(pend->r2));
                            split_read_store(pend->r1, n, drop);
                            split_read_store(pend->r2, n, drop);
                            at_end = true;
                        }
                    } else {
                        k1 = p1->parse(pend->r1, step);
                    }
                    if (k1 < step) at_end = true;
                }
                const size_t n = read_store_size(pend->r1);
                if (n == 0) break;
                pend->records = records;
                auto next = std::make_unique<InBatch>();
                split_read_store(pend->r1, cut, next->r1);
                if (p2) split_read_store(pend->r2, cut, next->r2);
                rec_est = std::max<size_t>(rec_est, n + n / 8);
                reserve(next->r1, rec_est);
                if (p2) reserve(next->r2, rec_est);
                if (!inq.push(std::move(pend))) break;
                pend = std::move(next);
                if (at_end && read_store_size(pend->r1) == 0) break;
            }
        } catch (...) {
            reader_err = std::current_exception();
        }
        inq.close();
    });

    std::thread writer([&] {
        try {
            if (cfg.header && cfg.header_len) {
                if (std::fwrite(cfg.header, 1, cfg.header_len, out) != cfg.header_len)
                    throw Error(SA_ERR_IO, "write error on " + out_path);
                bytes_out += cfg.header_len;
            }
            sa_output o;
            while (outq.pop(o)) {
                const bool ok = o.len == 0 || std::fwrite(o.data, 1, o.len, out) == o.len;
                bytes_out += o.len;
                release_output(o.data);
                if (!ok) throw Error(SA_ERR_IO, "write error on " + out_path);
            }
        } catch (...) {
            writer_err = std::current_exception();
            sa_output o;
            while (outq.pop(o)) release_output(o.data);
        }
    });

    std::exception_ptr map_err;
    try {
        for (;;) {
            const auto tw = std::chrono::steady_clock::now();
            std::unique_ptr<InBatch> b;
            const bool got = inq.pop(b);
            res.seconds_wait_input += since(tw);
            if (!got) break;
            const sa_read_batch v1 = view_of(b->r1);
            const sa_read_batch v2 = p2 ? view_of(b->r2) : sa_read_batch{};
            sa_output o{};
            const auto tm = std::chrono::steady_clock::now();
            if (cfg.interleaved) m.map_interleaved(&v1, &o);
            else m.map(&v1, p2 ? &v2 : nullptr, &o);
            res.seconds_map += since(tm);
            res.records += b->records;
            res.reads += o.n_reads;
            res.mapped += o.n_mapped;
            res.batches++;
            b.reset();
            if (!outq.push(std::move(o))) {
                release_output(o.data);
                break;
            }
            if (writer_err) break;
        }
    } catch (...) {
        map_err = std::current_exception();
    }
    inq.close();  // stops the reader if mapping ended early
    reader.join();
    outq.close();
    writer.join();
    std::exception_ptr err = map_err ? map_err : writer_err ? writer_err : reader_err;
    if (!err) {
        try {
            if (m.mapping_params().mode == SA_MODE_ABUNDANCE) {
                // output_abundances (src/main.rs:990-1001): name, abundance / length
                const auto& ab = m.abundances();
                const auto& cs = m.contigs();
                for (size_t i = 0; i < cs.size(); i++) {
                    const int k = std::fprintf(out, "%s\t%.6f\n", cs[i].name->c_str(), ab[i] / (double)cs[i].len);
                    if (k < 0) throw Error(SA_ERR_IO, "write error on " + out_path);
                    bytes_out += (uint64_t)k;
                }
            }
            if (std::fflush(out) != 0) throw Error(SA_ERR_IO, "write error on " + out_path);
        } catch (...) {
            err = std::current_exception();
        }
    }
    close_out();
    if (err) std::rethrow_exception(err);
    res.bytes_in = p1->file_bytes() + (p2 ? p2->file_bytes() : 0);
    res.bytes_out = bytes_out;
    res.seconds_total = since(t0);
    return res;
}

}  // namespace sa
