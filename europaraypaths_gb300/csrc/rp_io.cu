// rp_io.cu -- the reference's text file formats (host code): parsers for the
// facet, target, source-path, gain, receive-window and attenuation-prism
// files and the per-trace output writer (src/CUDA/file_io.cu:284-624).
//
// Differences from the reference, all deliberate:
//   * values are parsed at full (double) precision; the reference stores them
//     as float;
//   * the number of records is the number of parsed lines; the reference
//     sizes its arrays by newline count + 1 (count_lines, file_io.cu:314-335),
//     which leaves one uninitialised record when a file ends with a newline;
//   * malformed records are errors (RP_ERR_PARSE, with file and line) instead
//     of a message and a silently truncated read.
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <dirent.h>
#include <string>
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>
#include <vector>

#include "rp_internal.h"

namespace {

struct File {
    FILE* f = nullptr;
    explicit File(const char* p) : f(p ? fopen(p, "r") : nullptr) {}
    ~File() { if (f) fclose(f); }
};

int check_file(const char* path) {
    struct stat sb;
    if (!path || stat(path, &sb) != 0) {
        rp_set_error("File not found: %s", path ? path : "(null)");
        return RP_ERR_IO;
    }
    if (!S_ISREG(sb.st_mode)) {
        rp_set_error("Not a regular file: %s", path);
        return RP_ERR_IO;
    }
    return RP_OK;
}

// Read all lines (without the newline); a final line without a newline counts.
int read_lines(const char* path, std::vector<std::string>& lines) {
    int rc = check_file(path);
    if (rc) return rc;
    File fl(path);
    if (!fl.f) { rp_set_error("Could not open %s: %s", path, strerror(errno)); return RP_ERR_IO; }
    std::string cur;
    char buf[1 << 16];
    size_t n;
    while ((n = fread(buf, 1, sizeof(buf), fl.f)) > 0) {
        for (size_t i = 0; i < n; ++i) {
            if (buf[i] == '\n') { lines.push_back(cur); cur.clear(); }
            else cur.push_back(buf[i]);
        }
    }
    if (!cur.empty()) lines.push_back(cur);
    return RP_OK;
}

bool blank(const std::string& s) {
    for (char c : s)
        if (c != ' ' && c != '\t' && c != '\r') return false;
    return true;
}

// Parse up to `n` numbers separated by any of `seps` (whitespace allowed).
int parse_numbers(const std::string& s, const char* seps, double* out, int n) {
    const char* p = s.c_str();
    int k = 0;
    while (*p && k < n) {
        while (*p == ' ' || *p == '\t') ++p;
        char* end = nullptr;
        double v = strtod(p, &end);
        if (end == p) return -1;
        out[k++] = v;
        p = end;
        while (*p == ' ' || *p == '\t' || *p == '\r') ++p;
        if (*p && strchr(seps, *p)) ++p;
        else break;
    }
    return k;
}

int count_char(const std::string& s, char c) {
    int k = 0;
    for (char x : s) k += (x == c);
    return k;
}

}  // namespace

// Number of records (non-blank lines) of a text file; count_lines,
// src/CUDA/file_io.cu:314-335 (see the note on trailing newlines above).
extern "C" int rp_count_records(const char* path, int64_t* n) {
    if (!n) { rp_set_error("rp_count_records: null argument"); return RP_ERR_ARG; }
    std::vector<std::string> lines;
    int rc = read_lines(path, lines);
    if (rc) return rc;
    int64_t k = 0;
    for (auto& l : lines) k += !blank(l);
    *n = k;
    return RP_OK;
}

// Facet file "x,y,z:nx,ny,nz:ux,uy,uz:vx,vy,vz" (loadFacetFile,
// file_io.cu:337-362) -> double[12][cap] SoA.
extern "C" int rp_read_facets(const char* path, double* soa, int64_t cap, int64_t* n) {
    if (!soa || !n || cap < 0) { rp_set_error("rp_read_facets: bad argument"); return RP_ERR_ARG; }
    std::vector<std::string> lines;
    int rc = read_lines(path, lines);
    if (rc) return rc;
    int64_t i = 0;
    for (size_t ln = 0; ln < lines.size(); ++ln) {
        if (blank(lines[ln])) continue;
        if (i >= cap) { rp_set_error("%s: more facets than the %lld allocated", path, (long long)cap); return RP_ERR_ARG; }
        double v[12];
        if (parse_numbers(lines[ln], ",:", v, 12) != 12) {
            rp_set_error("%s line %zu: expected 12 numbers 'x,y,z:nx,ny,nz:ux,uy,uz:vx,vy,vz'", path, ln + 1);
            return RP_ERR_PARSE;
        }
        for (int c = 0; c < 12; ++c) soa[(size_t)c * cap + i] = v[c];
        ++i;
    }
    *n = i;
    return RP_OK;
}

// Target file with 3, 4, 6 or 7 comma-separated columns (loadTargetFile,
// file_io.cu:365-426): default normal +z, default ttype 0 -> double[7][cap].
extern "C" int rp_read_targets(const char* path, double* soa, int64_t cap, int64_t* n) {
    if (!soa || !n || cap < 0) { rp_set_error("rp_read_targets: bad argument"); return RP_ERR_ARG; }
    std::vector<std::string> lines;
    int rc = read_lines(path, lines);
    if (rc) return rc;
    int64_t i = 0;
    for (size_t ln = 0; ln < lines.size(); ++ln) {
        if (blank(lines[ln])) continue;
        if (i >= cap) { rp_set_error("%s: more targets than the %lld allocated", path, (long long)cap); return RP_ERR_ARG; }
        const int commas = count_char(lines[ln], ',');
        double v[7] = {0, 0, 0, 0, 0, 1, 0};
        int want = commas + 1;
        if (commas != 2 && commas != 3 && commas != 5 && commas != 6) {
            rp_set_error("Error: Target file line number=%zu has incorrect number of entries.", ln + 1);
            return RP_ERR_PARSE;
        }
        double t[7];
        if (parse_numbers(lines[ln], ",", t, want) != want) {
            rp_set_error("%s line %zu: malformed number", path, ln + 1);
            return RP_ERR_PARSE;
        }
        v[0] = t[0]; v[1] = t[1]; v[2] = t[2];
        if (want == 4) v[6] = t[3];
        if (want >= 6) { v[3] = t[3]; v[4] = t[4]; v[5] = t[5]; }
        if (want == 7) v[6] = t[6];
        // %hhu: the type is an unsigned char
        v[6] = (double)((unsigned)(long long)v[6] & 0xffu);
        for (int c = 0; c < 7; ++c) soa[(size_t)c * cap + i] = v[c];
        ++i;
    }
    *n = i;
    return RP_OK;
}

// Source-path file with 3 or 6 columns (loadSourceFile, file_io.cu:429-474)
// -> rows of 6: x,y,z, nx,ny,nz (default normal +z).
extern "C" int rp_read_sources(const char* path, double* rows, int64_t cap, int64_t* n) {
    if (!rows || !n || cap < 0) { rp_set_error("rp_read_sources: bad argument"); return RP_ERR_ARG; }
    std::vector<std::string> lines;
    int rc = read_lines(path, lines);
    if (rc) return rc;
    int64_t i = 0;
    for (size_t ln = 0; ln < lines.size(); ++ln) {
        if (blank(lines[ln])) continue;
        if (i >= cap) { rp_set_error("%s: more sources than the %lld allocated", path, (long long)cap); return RP_ERR_ARG; }
        const int commas = count_char(lines[ln], ',');
        if (commas != 2 && commas != 5) {
            rp_set_error("Error: Source file line number=%zu has incorrect number of entries.", ln + 1);
            return RP_ERR_PARSE;
        }
        double t[6] = {0, 0, 0, 0, 0, 1};
        if (parse_numbers(lines[ln], ",", t, commas + 1) != commas + 1) {
            rp_set_error("%s line %zu: malformed number", path, ln + 1);
            return RP_ERR_PARSE;
        }
        for (int c = 0; c < 6; ++c) rows[6 * i + c] = t[c];
        ++i;
    }
    *n = i;
    return RP_OK;
}

// Gain-pattern file "surface_dB,subsurface_dB" per line, blank lines skipped
// (loadGainFile, file_io.cu:597-624) -> rows of 2.
extern "C" int rp_read_gains(const char* path, double* rows, int64_t cap, int64_t* n) {
    if (!rows || !n || cap < 0) { rp_set_error("rp_read_gains: bad argument"); return RP_ERR_ARG; }
    std::vector<std::string> lines;
    int rc = read_lines(path, lines);
    if (rc) return rc;
    int64_t i = 0;
    for (size_t ln = 0; ln < lines.size(); ++ln) {
        if (blank(lines[ln])) continue;
        if (i >= cap) { rp_set_error("%s: more gain entries than the %lld allocated", path, (long long)cap); return RP_ERR_ARG; }
        double t[2];
        if (parse_numbers(lines[ln], ",", t, 2) != 2) {
            rp_set_error("%s line %zu: expected 'surface_gain,subsurface_gain'", path, ln + 1);
            return RP_ERR_PARSE;
        }
        rows[2 * i] = t[0];
        rows[2 * i + 1] = t[1];
        ++i;
    }
    *n = i;
    return RP_OK;
}

// Receive-window start positions, one number per line, exactly ns lines
// (loadRxWindowPositions, file_io.cu:520-551; the reference exits otherwise).
extern "C" int rp_read_rx_window(const char* path, double* out, int64_t ns) {
    if (!out || ns < 0) { rp_set_error("rp_read_rx_window: bad argument"); return RP_ERR_ARG; }
    std::vector<std::string> lines;
    int rc = read_lines(path, lines);
    if (rc) return rc;
    int64_t i = 0;
    for (size_t ln = 0; ln < lines.size(); ++ln) {
        if (blank(lines[ln])) continue;
        if (i >= ns) {
            rp_set_error("Error: rx_window_positions file has MORE entries than sources (ns = %lld)", (long long)ns);
            return RP_ERR_PARSE;
        }
        double t;
        if (parse_numbers(lines[ln], ",", &t, 1) != 1) {
            rp_set_error("Error: Invalid float on line %lld", (long long)(i + 1));
            return RP_ERR_PARSE;
        }
        out[i++] = t;
    }
    if (i != ns) {
        rp_set_error("Error: rx_window_positions file has %lld entries, but expected exactly %lld",
                     (long long)i, (long long)ns);
        return RP_ERR_PARSE;
    }
    return RP_OK;
}

// Attenuation prisms "sigma,xmin,ymin,zmin,xmax,ymax,zmax" (loadAttenPrismFile,
// file_io.cu:477-517) -> double[7][cap] with sigma turned into alpha.
extern "C" int rp_prism_alpha(const rp_params* p, double conductivity, double* alpha);

extern "C" int rp_read_prisms(const char* path, const rp_params* p, double* soa, int64_t cap, int64_t* n) {
    if (!p || !soa || !n || cap < 0) { rp_set_error("rp_read_prisms: bad argument"); return RP_ERR_ARG; }
    std::vector<std::string> lines;
    int rc = read_lines(path, lines);
    if (rc) return rc;
    int64_t i = 0;
    for (size_t ln = 0; ln < lines.size(); ++ln) {
        if (blank(lines[ln])) continue;
        if (i >= cap) { rp_set_error("%s: more attenuation prisms than the %lld allocated", path, (long long)cap); return RP_ERR_ARG; }
        double t[7];
        if (parse_numbers(lines[ln], ",", t, 7) != 7) {
            rp_set_error("%s line %zu: expected 'sigma,xmin,ymin,zmin,xmax,ymax,zmax'", path, ln + 1);
            return RP_ERR_PARSE;
        }
        double a;
        if ((rc = rp_prism_alpha(p, t[0], &a))) return rc;
        soa[i] = a;
        for (int c = 1; c < 7; ++c) soa[(size_t)c * cap + i] = t[c];
        ++i;
    }
    *n = i;
    return RP_OK;
}

// One trace as "%e %e\n" per bin (saveSignalToFile, file_io.cu:284-296).
extern "C" int rp_write_trace(const char* path, const float* re_im, int64_t nr) {
    if (!path || !re_im || nr < 0) { rp_set_error("rp_write_trace: bad argument"); return RP_ERR_ARG; }
    FILE* f = fopen(path, "w");
    if (!f) { rp_set_error("Could not write %s: %s", path, strerror(errno)); return RP_ERR_IO; }
    for (int64_t i = 0; i < nr; ++i) fprintf(f, "%e %e\n", (double)re_im[2 * i], (double)re_im[2 * i + 1]);
    int bad = ferror(f);
    fclose(f);
    if (bad) { rp_set_error("write error on %s", path); return RP_ERR_IO; }
    return RP_OK;
}

// The output directory must exist (checkDirectoryExists, file_io.cu:266-281).
extern "C" int rp_check_directory(const char* path) {
    struct stat sb;
    if (!path || stat(path, &sb) != 0) {
        rp_set_error("Directory not found: %s", path ? path : "(null)");
        return RP_ERR_IO;
    }
    if (!S_ISDIR(sb.st_mode)) {
        rp_set_error("Path is not a directory: %s", path);
        return RP_ERR_IO;
    }
    return RP_OK;
}

// Remove s*.txt from a directory (remove_s_txt_files, file_io.cu:554-593).
extern "C" int rp_clear_traces(const char* dir, int64_t* removed) {
    int rc = rp_check_directory(dir);
    if (rc) return rc;
    DIR* dp = opendir(dir);
    if (!dp) { rp_set_error("Invalid directory %s", dir); return RP_ERR_IO; }
    int64_t k = 0;
    struct dirent* e;
    while ((e = readdir(dp)) != nullptr) {
        std::string name(e->d_name);
        if (name.size() < 5 || name[0] != 's' || name.substr(name.size() - 4) != ".txt") continue;
        std::string full = std::string(dir) + "/" + name;
        if (unlink(full.c_str()) == 0) ++k;
    }
    closedir(dp);
    if (removed) *removed = k;
    return RP_OK;
}

// ------------------------------------------------------------ binary store --
// The binary replacements of the text formats: one 32-byte header (8-byte
// magic, record count, column or bin count, element kind), then the data in
// exactly the in-memory layout of the C ABI, so a store is memory-mapped and
// handed to rp_scene_create without parsing or copying on the host:
//   facets  "RPFCT01\0"  n, 12, 0   float64 SoA [12][n]
//   targets "RPTGT01\0"  n,  7, 0   float64 SoA [7][n]
//   radargram "RPRDR01\0" ns, nr, k  k = 0 complex64, 1 complex128, [ns][nr]
// Header fields are little-endian int64, as on both supported hosts.
namespace {

const char kMagic[3][8] = {{'R', 'P', 'F', 'C', 'T', '0', '1', 0},
                           {'R', 'P', 'T', 'G', 'T', '0', '1', 0},
                           {'R', 'P', 'R', 'D', 'R', '0', '1', 0}};
const int64_t kCols[2] = {12, 7};

struct Header {
    char magic[8];
    int64_t n, m, kind;
};
static_assert(sizeof(Header) == 32, "binary store header is 32 bytes");

struct Map {        // one read-only mapping of a store file
    void* base;
    size_t bytes;
};

int write_all(const char* path, const Header& h, const void* data, size_t bytes) {
    FILE* f = fopen(path, "wb");
    if (!f) { rp_set_error("Could not write %s: %s", path, strerror(errno)); return RP_ERR_IO; }
    bool ok = fwrite(&h, sizeof(h), 1, f) == 1;
    if (ok && bytes) ok = fwrite(data, 1, bytes, f) == bytes;
    ok = (fclose(f) == 0) && ok;
    if (!ok) { rp_set_error("write error on %s", path); return RP_ERR_IO; }
    return RP_OK;
}

int read_header(const char* path, int which, Header* h, size_t* file_bytes) {
    int rc = check_file(path);
    if (rc) return rc;
    File fl(path);
    if (!fl.f) { rp_set_error("Could not open %s: %s", path, strerror(errno)); return RP_ERR_IO; }
    if (fread(h, sizeof(*h), 1, fl.f) != 1) { rp_set_error("%s: shorter than a store header", path); return RP_ERR_PARSE; }
    if (memcmp(h->magic, kMagic[which], 8) != 0) { rp_set_error("%s: not a %s store", path,
        which == 0 ? "facet" : (which == 1 ? "target" : "radargram")); return RP_ERR_PARSE; }
    struct stat sb;
    stat(path, &sb);
    *file_bytes = (size_t)sb.st_size;
    return RP_OK;
}

}  // namespace

// Whether a file starts with a binary store header: 0 facets, 1 targets,
// 2 radargram, -1 anything else (a text file).
extern "C" int rp_store_kind(const char* path, int* kind) {
    if (!path || !kind) { rp_set_error("rp_store_kind: null argument"); return RP_ERR_ARG; }
    int rc = check_file(path);
    if (rc) return rc;
    File fl(path);
    char m[8];
    *kind = -1;
    if (fl.f && fread(m, 1, 8, fl.f) == 8)
        for (int k = 0; k < 3; ++k)
            if (memcmp(m, kMagic[k], 8) == 0) *kind = k;
    return RP_OK;
}

// Write a facet (kind 0, 12 columns) or target (kind 1, 7 columns) SoA store.
extern "C" int rp_write_store(const char* path, int kind, const double* soa, int64_t n) {
    if (!path || (kind != 0 && kind != 1) || n < 0 || (n > 0 && !soa)) {
        rp_set_error("rp_write_store: bad argument");
        return RP_ERR_ARG;
    }
    Header h;
    memcpy(h.magic, kMagic[kind], 8);
    h.n = n; h.m = kCols[kind]; h.kind = 0;
    return write_all(path, h, soa, sizeof(double) * (size_t)kCols[kind] * (size_t)n);
}

// Memory-map a facet or target store read-only: *soa points at its [cols][n]
// float64 data, valid until rp_unmap_store(*handle).
extern "C" int rp_map_store(const char* path, int kind, const double** soa, int64_t* n, void** handle) {
    if (!path || (kind != 0 && kind != 1) || !soa || !n || !handle) {
        rp_set_error("rp_map_store: bad argument");
        return RP_ERR_ARG;
    }
    Header h;
    size_t fb = 0;
    int rc = read_header(path, kind, &h, &fb);
    if (rc) return rc;
    if (h.n < 0 || h.m != kCols[kind] || h.kind != 0 ||
        fb != sizeof(Header) + sizeof(double) * (size_t)h.m * (size_t)h.n) {
        rp_set_error("%s: header (n %lld, columns %lld) does not match the file size %zu", path,
                     (long long)h.n, (long long)h.m, fb);
        return RP_ERR_PARSE;
    }
    int fd = open(path, O_RDONLY);
    if (fd < 0) { rp_set_error("Could not open %s: %s", path, strerror(errno)); return RP_ERR_IO; }
    void* base = mmap(nullptr, fb, PROT_READ, MAP_PRIVATE, fd, 0);
    close(fd);
    if (base == MAP_FAILED) { rp_set_error("mmap of %s failed: %s", path, strerror(errno)); return RP_ERR_IO; }
    Map* m = new Map{base, fb};
    *soa = reinterpret_cast<const double*>(static_cast<const char*>(base) + sizeof(Header));
    *n = h.n;
    *handle = m;
    return RP_OK;
}

extern "C" int rp_unmap_store(void* handle) {
    if (!handle) return RP_OK;
    Map* m = static_cast<Map*>(handle);
    munmap(m->base, m->bytes);
    delete m;
    return RP_OK;
}

// The whole radargram as one file: ns traces of nr complex64 (complex128 = 0)
// or complex128 (complex128 = 1) values, trace-major.
extern "C" int rp_write_radargram(const char* path, const void* data, int64_t ns, int64_t nr, int complex128) {
    if (!path || ns < 0 || nr < 0 || (ns * nr > 0 && !data)) {
        rp_set_error("rp_write_radargram: bad argument");
        return RP_ERR_ARG;
    }
    Header h;
    memcpy(h.magic, kMagic[2], 8);
    h.n = ns; h.m = nr; h.kind = complex128 ? 1 : 0;
    return write_all(path, h, data, (size_t)ns * (size_t)nr * (complex128 ? 16 : 8));
}

// Shape and element kind of a radargram file.
extern "C" int rp_radargram_info(const char* path, int64_t* ns, int64_t* nr, int* complex128) {
    if (!path || !ns || !nr || !complex128) { rp_set_error("rp_radargram_info: null argument"); return RP_ERR_ARG; }
    Header h;
    size_t fb = 0;
    int rc = read_header(path, 2, &h, &fb);
    if (rc) return rc;
    const size_t es = h.kind == 1 ? 16 : 8;
    if (h.n < 0 || h.m < 0 || (h.kind != 0 && h.kind != 1) || fb != sizeof(Header) + (size_t)h.n * (size_t)h.m * es) {
        rp_set_error("%s: radargram header does not match the file size", path);
        return RP_ERR_PARSE;
    }
    *ns = h.n; *nr = h.m; *complex128 = (int)h.kind;
    return RP_OK;
}

// Read a radargram file into data (ns x nr of the file's element kind).
extern "C" int rp_read_radargram(const char* path, void* data, int64_t ns, int64_t nr, int complex128) {
    int64_t fns, fnr;
    int fk;
    int rc = rp_radargram_info(path, &fns, &fnr, &fk);
    if (rc) return rc;
    if (!data || fns != ns || fnr != nr || fk != (complex128 ? 1 : 0)) {
        rp_set_error("rp_read_radargram: the buffer does not match %s", path);
        return RP_ERR_ARG;
    }
    File fl(path);
    const size_t bytes = (size_t)ns * (size_t)nr * (fk ? 16 : 8);
    if (fseek(fl.f, (long)sizeof(Header), SEEK_SET) != 0 || (bytes && fread(data, 1, bytes, fl.f) != bytes)) {
        rp_set_error("read error on %s", path);
        return RP_ERR_IO;
    }
    return RP_OK;
}
