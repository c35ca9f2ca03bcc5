// Text files of the reference's on-disk formats: the OpenFOAM LDU matrix,
// vector and processor-interface dumps that
// tools/readData/readFromOpenFOAM/readFromOpenFOAM.cpp reads and
// tools/printData/printUNAP/printUNAP.cpp writes.
//
// Formats (one record per line, fields separated by white space):
//   matrix     "nCells: N nnz: M symm: s", then N lines "i i diag" and
//              nFaces lines "l u upper [lower]", nFaces = M - N when s != 0,
//              else (M - N) / 2 (readFromOpenFOAM.cpp:26-59)
//   vector     "nCells: N", then N lines whose first field is the value
//              (readFromOpenFOAM.cpp:142-204)
//   interfaces header with nNeiProcs in field 2 and the total face count in
//              field 5; per neighbour a line with its rank in field 1 and
//              its face count in field 3, then one "faceCell coeff" line
//              per face; coefficients are stored negated
//              (readFromOpenFOAM.cpp:207-322)
//
// Field semantics follow the reference reader exactly: lines are split at
// '\n' like std::getline, fields at C-locale white space like
// `istringstream >> string`, a real field is converted like atof and an
// integer field like atoi.  Reals are parsed with std::from_chars, which
// rounds correctly like glibc's strtod, and any field from_chars does not
// consume whole (a leading '+', hex floats, trailing garbage, overflow) goes
// to strtod/strtol themselves, so every value is bit-identical to atof/atoi.
// The printers write "%.15e" like the reference's
// `setiosflags(ios::scientific) << setprecision(15)` through std::to_chars,
// whose exact shortest-digit algorithm rounds ties to even like glibc's
// printf, so the files are byte-identical.
//
// Both directions split the file into byte ranges and work on them from a
// pool of host threads: a 10-million-line dump parses in a fraction of a
// second instead of the reference's per-line stringstreams.
//
// Deliberate differences, each an error return instead of undefined
// behaviour in the reference: an unreadable or empty file; a data line with
// fewer fields than the reference reads (it would leave that entry
// uninitialised); sizes that are negative or overflow 32-bit indices.
#include <algorithm>
#include <cerrno>
#include <charconv>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "../../include/unap_cuda.h"
#include "capi_handles.hpp"
#include "unap_internal.hpp"

namespace unapgpu {
namespace {

// ---------------------------------------------------------------- threads

int io_threads(size_t bytes)
{
    unsigned hw = std::thread::hardware_concurrency();
    if (hw == 0) hw = 1;
    size_t byWork = bytes / (size_t)(1 << 20) + 1;  // about 1 MB per thread at least
    size_t t = std::min<size_t>({(size_t)hw, (size_t)32, byWork});
    if (const char* e = std::getenv("UNAP_IO_THREADS")) {
        int v = std::atoi(e);
        if (v > 0) t = (size_t)v;
    }
    return (int)std::max<size_t>(1, t);
}

template <class F>
void parallel_for(int nt, F&& f)
{
    if (nt <= 1) {
        f(0);
        return;
    }
    std::vector<std::thread> th;
    std::vector<std::exception_ptr> err((size_t)nt);
    th.reserve((size_t)nt);
    for (int t = 0; t < nt; ++t)
        th.emplace_back([&, t] {
            try {
                f(t);
            } catch (...) {
                err[(size_t)t] = std::current_exception();
            }
        });
    for (auto& x : th) x.join();
    for (auto& e : err)
        if (e) std::rethrow_exception(e);
}

// ------------------------------------------------------------------ input

struct TextFile {
    std::string data;  // NUL-terminated by std::string
    std::string name;
};

TextFile slurp(const char* path)
{
    if (!path) throw std::invalid_argument("null file name");
    TextFile f;
    f.name = path;
    FILE* fp = std::fopen(path, "rb");
    if (!fp) throw std::invalid_argument("cannot open " + f.name);
    std::fseek(fp, 0, SEEK_END);
    long sz = std::ftell(fp);
    std::fseek(fp, 0, SEEK_SET);
    if (sz < 0) {
        std::fclose(fp);
        throw std::invalid_argument("cannot read " + f.name);
    }
    f.data.resize((size_t)sz);
    size_t got = sz ? std::fread(&f.data[0], 1, (size_t)sz, fp) : 0;
    std::fclose(fp);
    if (got != (size_t)sz) throw std::invalid_argument("short read of " + f.name);
    if (sz == 0) throw std::invalid_argument(f.name + " is empty");
    return f;
}

inline bool is_space(char c)
{
    // the C locale's isspace set, which `istringstream >> string` splits on
    return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r';
}

// Line starts, numbered like the vector std::getline fills: a line begins
// at offset 0 and after every '\n' that is not the last byte.
struct LineIndex {
    size_t nLines = 0;
    std::vector<size_t> chunkBegin;  // byte ranges, one per thread
    std::vector<size_t> firstLine;   // index of the first line starting in each range
    std::vector<size_t> firstStart;  // its byte offset (== range end if none)
};

LineIndex index_lines(const std::string& d, int nt)
{
    const size_t n = d.size();
    LineIndex L;
    L.chunkBegin.resize((size_t)nt + 1);
    for (int t = 0; t <= nt; ++t) L.chunkBegin[(size_t)t] = n * (size_t)t / (size_t)nt;
    std::vector<size_t> nl((size_t)nt, 0);
    parallel_for(nt, [&](int t) {
        const char* p = d.data() + L.chunkBegin[(size_t)t];
        const char* e = d.data() + L.chunkBegin[(size_t)t + 1];
        size_t c = 0;
        while ((p = (const char*)std::memchr(p, '\n', (size_t)(e - p)))) {
            ++c;
            ++p;
        }
        nl[(size_t)t] = c;
    });
    // a line starts at s when s == 0 or d[s-1] == '\n' (and s < n)
    L.firstLine.resize((size_t)nt);
    L.firstStart.resize((size_t)nt);
    size_t before = 0;  // '\n' bytes in [0, chunkBegin[t])
    for (int t = 0; t < nt; ++t) {
        size_t a = L.chunkBegin[(size_t)t], b = L.chunkBegin[(size_t)t + 1];
        size_t s = a;
        if (a > 0 && d[a - 1] != '\n') {
            const void* q = std::memchr(d.data() + a, '\n', b - a);
            s = q ? (size_t)((const char*)q - d.data()) + 1 : b;
        }
        L.firstStart[(size_t)t] = std::min(s, b);
        // lines before s = '\n' bytes in [0, s)
        L.firstLine[(size_t)t] = before + (s > a ? 1 : 0);
        before += nl[(size_t)t];
    }
    L.nLines = before + (d[n - 1] == '\n' ? 0 : 1);
    return L;
}

// the fields of one line [p, e)
struct Fields {
    static constexpr int kMax = 6;
    const char* f[kMax];
    int n = 0;  // fields seen (capped at kMax; the reader ignores extra ones)
};

inline const char* split_line(const char* p, const char* end, Fields& F)
{
    F.n = 0;
    while (p < end && *p != '\n') {
        if (is_space(*p)) {
            ++p;
            continue;
        }
        if (F.n < Fields::kMax) F.f[F.n] = p;
        ++F.n;
        while (p < end && *p != '\n' && !is_space(*p)) ++p;
    }
    if (F.n > Fields::kMax) F.n = Fields::kMax;
    return p < end ? p + 1 : end;  // past the '\n'
}

inline const char* field_end(const char* p)
{
    while (*p && !is_space(*p)) ++p;
    return p;
}

// atof(field): the buffer is NUL-terminated and fields end at white space,
// which no number can contain, so strtod on the buffer reads the same prefix
// atof reads from the field's own string.
inline double to_real(const char* p)
{
    const char* e = field_end(p);
    double v;
    auto r = std::from_chars(p, e, v);
    if (r.ec == std::errc() && r.ptr == e) return v;
    return std::strtod(p, nullptr);
}

// atoi(field) == (int) strtol(field, NULL, 10) in glibc
inline long to_long(const char* p)
{
    const char* e = field_end(p);
    long v;
    auto r = std::from_chars(p, e, v);
    if (r.ec == std::errc() && r.ptr == e) return (long)(int)v;
    return (long)(int)std::strtol(p, nullptr, 10);
}

const char* line_ptr_after_header(const std::string& d)
{
    const char* q = (const char*)std::memchr(d.data(), '\n', d.size());
    return q ? q + 1 : d.data() + d.size();
}

[[noreturn]] void short_line(const TextFile& f, size_t line, int want)
{
    throw std::invalid_argument(f.name + ": line " + std::to_string(line + 1) + " has fewer than " +
                                std::to_string(want) + " fields");
}

// Calls body(lineIndex, fields) for lines [first, first + count) of f, from
// nt threads.  Lines are numbered from the header (line 0).
template <class Body>
void for_lines(const TextFile& f, const LineIndex& L, int nt, size_t first, size_t count,
               Body&& body)
{
    const std::string& d = f.data;
    const size_t last = first + count;
    parallel_for(nt, [&](int t) {
        size_t line = L.firstLine[(size_t)t];
        const char* p = d.data() + L.firstStart[(size_t)t];
        const char* e = d.data() + L.chunkBegin[(size_t)t + 1];
        const char* end = d.data() + d.size();
        Fields F;
        while (p < e) {  // lines that start inside this range
            const char* next = split_line(p, end, F);
            if (line >= first && line < last) body(line, F);
            ++line;
            p = next;
        }
    });
}

// ----------------------------------------------------------------- output

struct OutBuf {
    std::vector<char> b;
    size_t n = 0;
    void reserve(size_t m) { b.resize(m); }
    char* room(size_t k)
    {
        if (n + k > b.size()) b.resize(std::max(b.size() * 2, n + k + 4096));
        return b.data() + n;
    }
    void put(const char* s, size_t k)
    {
        std::memcpy(room(k), s, k);
        n += k;
    }
    void put(char c) { *room(1) = c, ++n; }
    void put_long(long v)
    {
        char* p = room(24);
        n += (size_t)(std::to_chars(p, p + 24, v).ptr - p);
    }
    // "%.15e"
    void put_e15(double v)
    {
        char* p = room(40);
        n += (size_t)(std::to_chars(p, p + 40, v, std::chars_format::scientific, 15).ptr - p);
    }
};

// "<name>_<rank>.txt" (printUNAP.hpp:10-13); one GPU is rank 0
std::string dump_name(const char* name)
{
    if (!name) throw std::invalid_argument("null file name");
    return std::string(name) + "_0.txt";
}

void write_parts(const std::string& path, const std::string& head, const std::vector<OutBuf>& parts)
{
    FILE* fp = std::fopen(path.c_str(), "wb");
    if (!fp) throw std::invalid_argument("cannot create " + path);
    bool ok = std::fwrite(head.data(), 1, head.size(), fp) == head.size();
    for (const OutBuf& o : parts)
        ok = ok && (o.n == 0 || std::fwrite(o.b.data(), 1, o.n, fp) == o.n);
    ok = (std::fclose(fp) == 0) && ok;
    if (!ok) throw std::runtime_error("write to " + path + " failed");
}

// Prints records [0, count) with put(i, buf) from nt threads, in order.
template <class Put>
std::vector<OutBuf> format_records(size_t count, size_t bytesPerRecord, Put&& put)
{
    int nt = io_threads(count * bytesPerRecord);
    if ((size_t)nt > count) nt = (int)std::max<size_t>(1, count);
    std::vector<OutBuf> parts((size_t)nt);
    parallel_for(nt, [&](int t) {
        size_t a = count * (size_t)t / (size_t)nt, b = count * (size_t)(t + 1) / (size_t)nt;
        OutBuf& o = parts[(size_t)t];
        o.reserve((b - a) * bytesPerRecord + 64);
        for (size_t i = a; i < b; ++i) put(i, o);
    });
    return parts;
}

int checked_int(long long v, const char* what)
{
    if (v < 0 || v > 0x7fffffffLL)
        throw std::invalid_argument(std::string(what) + " out of range: " + std::to_string(v));
    return (int)v;
}

}  // namespace

// ------------------------------------------------------------ the formats

// constructLDUMatrixFromOpenFOAM (readFromOpenFOAM.cpp:9-139)
HostLdu read_ldu_text(const char* path)
{
    TextFile f = slurp(path);
    const int nt = io_threads(f.data.size());
    LineIndex L = index_lines(f.data, nt);

    // header fields 1, 3, 5: nCells, nnz, symm (readFromOpenFOAM.cpp:26-50)
    long nCells = -1, nnz = -1, symm = 0;
    {
        Fields F;
        split_line(f.data.data(), f.data.data() + f.data.size(), F);
        if (F.n > 1) nCells = to_long(F.f[1]);
        if (F.n > 3) nnz = to_long(F.f[3]);
        if (F.n > 5) symm = to_long(F.f[5]);
    }
    long nFaces = symm ? nnz - nCells : (nnz - nCells) / 2;
    if ((long long)L.nLines != (long long)nCells + nFaces + 1)
        throw std::invalid_argument("Error in reading " + f.name + ": reading " +
                                    std::to_string((long long)L.nLines - 1) +
                                    " lines, while nCells = " + std::to_string(nCells) +
                                    ", nFaces = " + std::to_string(nFaces));
    HostLdu h;
    h.n = checked_int(nCells, "nCells");
    h.nf = checked_int(nFaces, "nFaces");
    h.symm = symm != 0;
    h.diag.resize((size_t)h.n);
    h.l.resize((size_t)h.nf);
    h.u.resize((size_t)h.nf);
    h.upper.resize((size_t)h.nf);
    if (!h.symm) h.lower.resize((size_t)h.nf);
    const size_t n = (size_t)h.n;
    for_lines(f, L, nt, 1, n + (size_t)h.nf, [&](size_t line, const Fields& F) {
        size_t i = line - 1;
        if (i < n) {
            if (F.n < 3) short_line(f, line, 3);
            h.diag[i] = to_real(F.f[2]);
        } else {
            size_t j = i - n;
            if (F.n < (h.symm ? 3 : 4)) short_line(f, line, h.symm ? 3 : 4);
            h.l[j] = (int)to_long(F.f[0]);
            h.u[j] = (int)to_long(F.f[1]);
            h.upper[j] = to_real(F.f[2]);
            if (!h.symm) h.lower[j] = to_real(F.f[3]);
        }
    });
    return h;
}

// constructVectorFromOpenFOAM (readFromOpenFOAM.cpp:142-204)
void read_vector_text(const char* path, long long n, double* v)
{
    TextFile f = slurp(path);
    const int nt = io_threads(f.data.size());
    LineIndex L = index_lines(f.data, nt);
    long nCells = -1;
    {
        Fields F;
        split_line(f.data.data(), f.data.data() + f.data.size(), F);
        if (F.n > 1) nCells = to_long(F.f[1]);
    }
    if ((long long)L.nLines != (long long)nCells + 1)
        throw std::invalid_argument("Error in reading " + f.name + ": reading " +
                                    std::to_string((long long)L.nLines - 1) +
                                    " lines, while nCells = " + std::to_string(nCells));
    if ((long long)nCells != n)
        throw std::invalid_argument("Error in " + f.name + ": fill size = " +
                                    std::to_string(nCells) + ", while allocated size = " +
                                    std::to_string(n));
    if (n > 0 && !v) throw std::invalid_argument("null vector");
    for_lines(f, L, nt, 1, (size_t)n, [&](size_t line, const Fields& F) {
        if (F.n < 1) short_line(f, line, 1);
        v[line - 1] = to_real(F.f[0]);
    });
}

struct TextInterfaces {
    std::vector<int> neighbour, size;
    std::vector<int> faceCells;
    std::vector<double> coeffs;
};

// constructLDUInterfacesFromOpenFOAM (readFromOpenFOAM.cpp:207-322)
TextInterfaces read_interfaces_text(const char* path)
{
    TextFile f = slurp(path);
    const int nt = io_threads(f.data.size());
    LineIndex L = index_lines(f.data, nt);
    long nNei = -1, nFaces = -1;
    {
        Fields F;
        split_line(f.data.data(), f.data.data() + f.data.size(), F);
        if (F.n > 2) nNei = to_long(F.f[2]);
        if (F.n > 5) nFaces = to_long(F.f[5]);
    }
    if ((long long)L.nLines != (long long)nFaces + nNei + 1)
        throw std::invalid_argument("Error in reading " + f.name + ":, reading " +
                                    std::to_string((long long)L.nLines - 1) +
                                    " lines, while nNeiProcs = " + std::to_string(nNei) +
                                    ", nFaces = " + std::to_string(nFaces));
    TextInterfaces I;
    const int np = checked_int(nNei, "nNeiProcs");
    checked_int(nFaces, "nFaces");
    I.neighbour.resize((size_t)np);
    I.size.resize((size_t)np);
    // the patch headers are sequential: each one says how many face lines follow
    const char* p = line_ptr_after_header(f.data);
    const char* end = f.data.data() + f.data.size();
    size_t line = 1;
    long long total = 0;
    for (int i = 0; i < np; ++i) {
        Fields F;
        const char* next = split_line(p, end, F);
        long nb = 0, sz = 0;  // the reference keeps the previous patch's values
        if (i > 0) nb = I.neighbour[(size_t)i - 1], sz = I.size[(size_t)i - 1];
        if (F.n > 1) nb = to_long(F.f[1]);
        if (F.n > 3) sz = to_long(F.f[3]);
        I.neighbour[(size_t)i] = (int)nb;
        I.size[(size_t)i] = checked_int(sz, "patch size");
        total += sz;
        if (total + i + 1 > nFaces + nNei)
            throw std::invalid_argument(f.name + ": patch " + std::to_string(i) +
                                        " runs past the end of the file");
        p = next;
        ++line;
        for (long j = 0; j < sz; ++j) {
            next = split_line(p, end, F);
            if (F.n < 2) short_line(f, line, 2);
            I.faceCells.push_back((int)to_long(F.f[0]));
            I.coeffs.push_back(-to_real(F.f[1]));
            p = next;
            ++line;
        }
    }
    return I;
}

// printLDUMatrix (printUNAP.cpp:8-58)
void write_ldu_text(const char* name, const HostLdu& h)
{
    const std::string path = dump_name(name);
    const size_t n = (size_t)h.n, nf = (size_t)h.nf;
    const long nnz = (long)n + (long)nf * (h.symm ? 1 : 2);
    std::string head = "nCells: " + std::to_string(h.n) + " nnz: " + std::to_string(nnz) +
                       " symm: " + (h.symm ? "1" : "0") + "\n";
    const double* lower = h.lowerPtr();
    auto parts = format_records(n + nf, h.symm ? 48 : 72, [&](size_t i, OutBuf& o) {
        if (i < n) {
            o.put_long((long)i);
            o.put(' ');
            o.put_long((long)i);
            o.put(' ');
            o.put_e15(h.diag[i]);
        } else {
            size_t f = i - n;
            o.put_long(h.l[f]);
            o.put(' ');
            o.put_long(h.u[f]);
            o.put(' ');
            o.put_e15(h.upper[f]);
            o.put(' ');
            if (!h.symm) o.put_e15(lower[f]);
        }
        o.put('\n');
    });
    write_parts(path, head, parts);
}

// printVector (printUNAP.hpp:27-42)
void write_vector_text(const char* name, long long n, const double* v)
{
    if (n < 0) throw std::invalid_argument("negative vector size");
    if (n > 0 && !v) throw std::invalid_argument("null vector");
    const std::string path = dump_name(name);
    std::string head = "nCells: " + std::to_string(n) + "\n";
    auto parts = format_records((size_t)n, 24, [&](size_t i, OutBuf& o) {
        o.put_e15(v[i]);
        o.put('\n');
    });
    write_parts(path, head, parts);
}

// printInterfaces (printUNAP.cpp:61-87)
void write_interfaces_text(const char* name, int nNei, const int* neighbour, const int* size,
                           const int* faceCells, const double* coeffs)
{
    if (nNei < 0) throw std::invalid_argument("negative interface count");
    const std::string path = dump_name(name);
    std::string head = "neighbor processors: " + std::to_string(nNei) + "\n";
    OutBuf o;
    size_t k = 0;
    for (int i = 0; i < nNei; ++i) {
        if (size[i] < 0) throw std::invalid_argument("negative patch size");
        o.put("processor: ", 11);
        o.put_long(neighbour[i]);
        o.put(" size: ", 7);
        o.put_long(size[i]);
        o.put('\n');
        for (int j = 0; j < size[i]; ++j, ++k) {
            o.put_long(faceCells[k]);
            o.put(' ');
            o.put_e15(coeffs[k]);
            o.put('\n');
        }
    }
    std::vector<OutBuf> parts;
    parts.push_back(std::move(o));
    write_parts(path, head, parts);
}

}  // namespace unapgpu

using namespace unapgpu;

namespace {

template <class F>
int guarded_io(F&& f)
{
    try {
        f();
        return UNAP_CUDA_OK;
    } catch (const std::bad_alloc&) {
        set_last_error("out of host memory");
        return UNAP_CUDA_ENOMEM;
    } catch (const std::invalid_argument& e) {
        set_last_error(e.what());
        return UNAP_CUDA_EINVAL;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return UNAP_CUDA_EINTERNAL;
    }
}

}  // namespace

extern "C" {

int unap_cuda_read_ldu_matrix(const char* fileName, long int* handle)
{
    return guarded_io([&] {
        if (!handle) throw std::invalid_argument("null handle pointer");
        auto m = std::make_unique<MatHandle>();
        m->pending = read_ldu_text(fileName);
        m->hasValues = true;
        *handle = reinterpret_cast<long int>(m.release());
    });
}

int unap_cuda_read_vector(const char* fileName, long long n, double* v)
{
    return guarded_io([&] { read_vector_text(fileName, n, v); });
}

int unap_cuda_read_interfaces(const char* fileName, int* nNeiProcs, long long* nFaces,
                              int* neighbour, int* size, int* faceCells, double* coeffs)
{
    return guarded_io([&] {
        TextInterfaces I = read_interfaces_text(fileName);
        size_t np = I.neighbour.size(), nf = I.faceCells.size();
        if (nNeiProcs) *nNeiProcs = (int)np;
        if (nFaces) *nFaces = (long long)nf;
        if (neighbour) std::memcpy(neighbour, I.neighbour.data(), np * sizeof(int));
        if (size) std::memcpy(size, I.size.data(), np * sizeof(int));
        if (faceCells) std::memcpy(faceCells, I.faceCells.data(), nf * sizeof(int));
        if (coeffs) std::memcpy(coeffs, I.coeffs.data(), nf * sizeof(double));
    });
}

int unap_cuda_print_ldu_matrix(long int handle, const char* name)
{
    return guarded_io([&] {
        MatHandle* h = mat_from(handle);
        if (!h->hasValues && !h->M) throw std::invalid_argument("matrix has no coefficients yet");
        write_ldu_text(name, h->M ? h->M->host : h->pending);
    });
}

int unap_cuda_print_vector(const char* name, long long n, const double* v)
{
    return guarded_io([&] { write_vector_text(name, n, v); });
}

int unap_cuda_print_interfaces(const char* name, int nNeiProcs, const int* neighbour,
                               const int* size, const int* faceCells, const double* coeffs)
{
    return guarded_io(
        [&] { write_interfaces_text(name, nNeiProcs, neighbour, size, faceCells, coeffs); });
}

}  // extern "C"
