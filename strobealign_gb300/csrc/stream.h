// File-to-file mapping with parsing, mapping and writing overlapped (stream.cpp)
#pragma once
#include <string>

#include "mapper.h"

namespace sa {

struct StreamConfig {
    uint64_t batch_bases = 0;  // nucleotides per mapped batch, cut at chunk ends; 0: 2^29
    uint32_t read_ahead = 2;   // parsed batches queued ahead of the mapper
    bool append = false;       // append to the output file instead of truncating it
    const char* header = nullptr;
    size_t header_len = 0;
    bool interleaved = false;  // reads1 holds mixed single-end and paired records
};

struct StreamResult {
    uint64_t reads = 0, records = 0, mapped = 0, batches = 0, bytes_in = 0, bytes_out = 0;
    double seconds_total = 0, seconds_map = 0, seconds_wait_input = 0;
};

// Maps reads1 (and reads2, paired-end) into out_path ("-": standard output).  The
// output bytes are those of sa_map_batch over all records of the input at once.
StreamResult map_files(Mapper& m, const std::string& reads1, const std::string* reads2, const std::string& out_path,
                       const StreamConfig& cfg);

}  // namespace sa
