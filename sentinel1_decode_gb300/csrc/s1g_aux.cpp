// Product sidecars: the index file (36-byte records, one per block of
// packets) and the annotation file (26-byte records, one per packet) that a
// Level-0 product keeps beside each measurement file.  Field layouts follow
// index_decoder / annotation_decoder (aux_decoding.cpp:61-118): big-endian
// bit fields read MSB first, like read_n_bits (decoding_utils.cpp:95-134).
// Host code only; the cross-check against the GPU indexer is in s1g_api.cu.
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/s1g.h"
#include "s1g_aux.h"

namespace s1g {

namespace {

uint64_t bits(const uint8_t* rec, int start, int n) {
    uint64_t v = 0;
    for (int k = 0; k < n; ++k) {
        const int b = start + k;
        v = (v << 1) | ((rec[b >> 3] >> (7 - (b & 7))) & 1u);
    }
    return v;
}

}  // namespace

// Reads fixed-size records.  The reference's loop (`while (!data.eof())`
// around a read of one record into a zero-filled buffer) yields one record
// more than the file holds complete: the zero-padded partial tail, or an
// all-zero record when the file ends on a boundary.  reference_tail adds it.
bool read_records(const char* path, int rec_size, bool reference_tail, std::vector<uint8_t>& out, int64_t& n) {
    FILE* f = path ? fopen(path, "rb") : nullptr;
    if (!f) return false;
    out.clear();
    uint8_t buf[1 << 16];
    size_t got;
    while ((got = fread(buf, 1, sizeof(buf), f)) > 0) out.insert(out.end(), buf, buf + got);
    const bool err = ferror(f) != 0;
    fclose(f);
    if (err) return false;
    n = (int64_t)(out.size() / (size_t)rec_size);
    if (reference_tail) {
        n += 1;
        out.resize((size_t)n * rec_size, 0);
    } else {
        out.resize((size_t)n * rec_size);
    }
    return true;
}

void parse_index_record(const uint8_t* r, s1g_index_record& x) {
    x.date_time = bits(r, 0, 64);
    x.time_delta = bits(r, 64, 64);
    x.data_size = (uint32_t)bits(r, 128, 32);
    x.unit_offset = (uint32_t)bits(r, 160, 32);
    x.byte_offset = bits(r, 192, 64);
    x.variable_flag = (uint32_t)bits(r, 256, 8);
    x.spare_data = (uint32_t)bits(r, 264, 24);
}

void parse_annotation_record(const uint8_t* r, s1g_annotation_record& x) {
    x.days_ul = (uint32_t)bits(r, 0, 16);
    x.milliseconds_ul = (uint32_t)bits(r, 16, 32);
    x.microseconds_ul = (uint32_t)bits(r, 48, 16);
    x.days_dl = (uint32_t)bits(r, 64, 16);
    x.milliseconds_dl = (uint32_t)bits(r, 80, 32);
    x.microseconds_dl = (uint32_t)bits(r, 112, 16);
    x.packet_length = (uint32_t)bits(r, 128, 16);
    x.num_transfer_frames = (uint32_t)bits(r, 144, 16);
    x.error_flag = (uint32_t)bits(r, 160, 8);
    x.bit_1_type = (uint32_t)bits(r, 168, 1);
    x.bit_2_type = (uint32_t)bits(r, 169, 2);
    x.bit_6_type = (uint32_t)bits(r, 171, 6);
    x.spare_field = (uint32_t)bits(r, 177, 8);
}

bool load_index(const char* path, bool reference_tail, std::vector<s1g_index_record>& out) {
    std::vector<uint8_t> raw;
    int64_t n = 0;
    if (!read_records(path, kIndexRecordBytes, reference_tail, raw, n)) return false;
    out.resize((size_t)n);
    for (int64_t i = 0; i < n; ++i) parse_index_record(raw.data() + i * kIndexRecordBytes, out[(size_t)i]);
    return true;
}

bool load_annotation(const char* path, bool reference_tail, std::vector<s1g_annotation_record>& out) {
    std::vector<uint8_t> raw;
    int64_t n = 0;
    if (!read_records(path, kAnnotationRecordBytes, reference_tail, raw, n)) return false;
    out.resize((size_t)n);
    for (int64_t i = 0; i < n; ++i) parse_annotation_record(raw.data() + i * kAnnotationRecordBytes, out[(size_t)i]);
    return true;
}

double annotation_time(const s1g_annotation_record& r) {
    // aux_decoding.cpp:132-145: seconds between the GPS (1980-01-06) and
    // MJD2000 epochs; the record's microseconds are never added (the
    // reference reads the absent key "microseconds", which is 0)
    const double epoch_difference = 7300 * 86400;
    return (double)((uint64_t)r.days_ul * 86400) + ((uint64_t)r.milliseconds_ul * 1e-3) + (0 * 1e-6) +
           epoch_difference;
}

bool map_file(const char* path, const void** data, size_t* n) {
    *data = nullptr;
    *n = 0;
    const int fd = open(path, O_RDONLY);
    if (fd < 0) return false;
    struct stat st;
    if (fstat(fd, &st) != 0 || !S_ISREG(st.st_mode)) {
        close(fd);
        return false;
    }
    const size_t len = (size_t)st.st_size;
    if (len > 0) {
        void* m = mmap(nullptr, len, PROT_READ, MAP_PRIVATE, fd, 0);
        if (m == MAP_FAILED) {
            close(fd);
            return false;
        }
        madvise(m, len, MADV_SEQUENTIAL);
        madvise(m, len, MADV_WILLNEED);
        *data = m;
    }
    close(fd);
    *n = len;
    return true;
}

void unmap_file(const void* data, size_t n) {
    if (data && n) munmap(const_cast<void*>(data), n);
}

}  // namespace s1g

extern "C" {

int s1g_read_index(const char* path, s1g_index_record* out, int64_t cap, int64_t* count, int reference_tail) {
    if (!path || !count) return S1G_E_INVALID_ARGUMENT;
    std::vector<s1g_index_record> v;
    if (!s1g::load_index(path, reference_tail != 0, v)) return S1G_E_IO;
    *count = (int64_t)v.size();
    if (out && cap >= (int64_t)v.size() && !v.empty()) std::memcpy(out, v.data(), v.size() * sizeof(v[0]));
    return S1G_OK;
}

int s1g_read_annotation(const char* path, s1g_annotation_record* out, int64_t cap, int64_t* count,
                        int reference_tail) {
    if (!path || !count) return S1G_E_INVALID_ARGUMENT;
    std::vector<s1g_annotation_record> v;
    if (!s1g::load_annotation(path, reference_tail != 0, v)) return S1G_E_IO;
    *count = (int64_t)v.size();
    if (out && cap >= (int64_t)v.size() && !v.empty()) std::memcpy(out, v.data(), v.size() * sizeof(v[0]));
    return S1G_OK;
}

int s1g_annotation_times(const char* path, double* out, int64_t cap, int64_t* count, int reference_tail) {
    if (!path || !count) return S1G_E_INVALID_ARGUMENT;
    std::vector<s1g_annotation_record> v;
    if (!s1g::load_annotation(path, reference_tail != 0, v)) return S1G_E_IO;
    *count = (int64_t)v.size();
    if (out && cap >= (int64_t)v.size())
        for (size_t i = 0; i < v.size(); ++i) out[i] = s1g::annotation_time(v[i]);
    return S1G_OK;
}

}  // extern "C"
