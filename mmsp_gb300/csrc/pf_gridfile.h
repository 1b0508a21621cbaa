// pf_gridfile.h -- MMSP grid files written from host memory (host code).
//
// The byte layout is the reference's grid::output (include/MMSP.grid.cpp:
// 1358-1402) with one block, as a serial run writes it (write_buffer,
// include/MMSP.grid.cpp:1818-1909):
//   ASCII header  "grid:<type>\n" "dim\n" "fields\n" ("g0 g1\n")*dim ("dx\n")*dim
//   int32 nblocks = 1
//   int32 x0,x1 per axis; int32 b0,b1 per axis; uint64 size_in_mem; uint64 size_on_disk
//   payload: to_buffer order (include/MMSP.grid.cpp:1146-1157), zlib-compressed
//            unless size_on_disk == size_in_mem (the reference's RAW form)
#pragma once

#include <stddef.h>

#include <string>

namespace pf {

struct GridFileInfo {
    int dim;
    int g0[3], n[3];   // global lower corner and extents per axis
    int bc[3][2];      // boundary codes per axis (include/MMSP.utility.h:23-29)
    double dx[3];
    int fields_line;   // the header's "fields" value
    bool vector;       // grid<dim,vector<T>>: each cell is int32 N + N values
    bool f64;          // double, else float
};

// Payload bytes of one grid in to_buffer order.
size_t payload_bytes(const GridFileInfo& fi, int fields);

// The ASCII header of grid::output.
std::string grid_header(const GridFileInfo& fi);

// Payloads up to this size are compressed by one compress2 call, exactly as
// the reference does; larger ones in independent chunks of this size.
constexpr size_t kDeflateChunk = 1u << 20;

// Write `payload` (size_in_mem bytes, to_buffer order) as an MMSP grid file.
// level 1..9: zlib level; 0: uncompressed (the reference's RAW form).
// threads <= 0: every hardware thread.  Returns MMSP_GPU_OK or a negative
// MMSP_GPU_E* code with the reason in *why.
int write_grid_file(const char* filename, const GridFileInfo& fi, const void* payload, size_t size_in_mem, int level,
                    int threads, std::string* why);

}  // namespace pf
