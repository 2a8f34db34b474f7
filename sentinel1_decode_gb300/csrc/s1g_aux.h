// Product sidecar readers shared by the C ABI and the cross-check of the
// GPU packet indexer (s1g_aux.cpp).
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

#include "../../include/s1g.h"

namespace s1g {

constexpr int kIndexRecordBytes = 36;        // aux_decoding.cpp:64
constexpr int kAnnotationRecordBytes = 26;   // aux_decoding.cpp:99

bool load_index(const char* path, bool reference_tail, std::vector<s1g_index_record>& out);
bool load_annotation(const char* path, bool reference_tail, std::vector<s1g_annotation_record>& out);
double annotation_time(const s1g_annotation_record& r);

// Map a regular file read-only (MAP_PRIVATE, sequential read-ahead).  An
// empty file maps to (nullptr, 0).  False if it cannot be opened or mapped.
bool map_file(const char* path, const void** data, size_t* n);
void unmap_file(const void* data, size_t n);

}  // namespace s1g
