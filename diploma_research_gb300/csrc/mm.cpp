// mm.cpp -- Matrix Market coordinate files to CSR behind the C ABI (dimgpu_mm_*), for C++ callers of
// dim::io::matrix_market::load_as_csr (include/dim/io/matrix_market.h:25-83) without scnlib.
//
// The reference reads the banner with mmio (libs/mmio/mmio.c), refuses anything but coordinate matrices
// (matrix_market.h:59-60), scans "row col [value]" entries with whitespace between them
// (matrix_market.h:38-42), makes the indices 0-based, gives pattern matrices the value 1.0, and builds the
// CSR with csr::from_coo (csr.h:42-77): entries visited in file order, each off-diagonal entry of a
// symmetric (or Hermitian) file followed by its mirror (coo.h:33-46), counted per row, scattered, then
// each row sorted by column.  The per-row sort here is stable, so entries with equal column indices in
// one row keep their file order (the reference's std::sort leaves their order unspecified).
// Host code only; failures return DIMGPU_ERR_INVALID_ARGUMENT (not a coordinate Matrix Market file, an
// entry that does not scan or lies outside the matrix) or DIMGPU_ERR_IO (the file cannot be read).
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cctype>
#include <cerrno>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <stdexcept>
#include <string>
#include <vector>

#include "internal.hpp"

namespace dimgpu {
namespace mm {
namespace {

struct io_error : std::runtime_error {
    using std::runtime_error::runtime_error;
};

struct csr_host {
    uint32_t rows = 0, cols = 0;
    std::vector<uint32_t> row_ptr, col;
    std::vector<double> val;
};

// The file's bytes (mapped read-only).
class mapped {
public:
    explicit mapped(const char* path) {
        const int fd = ::open(path, O_RDONLY);
        if (fd < 0)
            throw io_error(std::string("cannot open ") + path + ": " + std::strerror(errno));
        struct stat st {};
        if (::fstat(fd, &st) != 0) {
            ::close(fd);
            throw io_error(std::string("cannot stat ") + path);
        }
        n_ = (size_t)st.st_size;
        if (n_) {
            void* p = ::mmap(nullptr, n_, PROT_READ, MAP_PRIVATE, fd, 0);
            if (p == MAP_FAILED) {
                ::close(fd);
                throw io_error(std::string("cannot map ") + path);
            }
            p_ = static_cast<const char*>(p);
        }
        ::close(fd);
    }
    ~mapped() {
        if (p_)
            ::munmap(const_cast<char*>(p_), n_);
    }
    mapped(const mapped&) = delete;
    mapped& operator=(const mapped&) = delete;
    const char* begin() const { return p_; }
    const char* end() const { return p_ + n_; }
    size_t size() const { return n_; }

private:
    const char* p_ = nullptr;
    size_t n_ = 0;
};

std::string lower(std::string s) {
    for (char& c : s)
        c = (char)std::tolower((unsigned char)c);
    return s;
}

// Reads whitespace-separated tokens from [p, end).
class scanner {
public:
    scanner(const char* p, const char* end) : p_(p), end_(end) {}
    const char* pos() const { return p_; }
    // the rest of the current line, advancing past its end
    std::string line() {
        const char* s = p_;
        while (p_ < end_ && *p_ != '\n')
            ++p_;
        std::string out(s, p_);
        if (p_ < end_)
            ++p_;
        if (!out.empty() && out.back() == '\r')
            out.pop_back();
        return out;
    }
    bool at_end() const { return p_ >= end_; }
    char peek() const { return p_ < end_ ? *p_ : '\0'; }
    void skip_space() {
        while (p_ < end_ && std::isspace((unsigned char)*p_))
            ++p_;
    }
    // the next token (empty at the end)
    std::string token() {
        skip_space();
        const char* s = p_;
        while (p_ < end_ && !std::isspace((unsigned char)*p_))
            ++p_;
        return std::string(s, p_);
    }

private:
    const char* p_;
    const char* end_;
};

uint64_t parse_index(const std::string& t) {
    if (t.empty())
        throw std::invalid_argument("scan failed");
    char* e = nullptr;
    errno = 0;
    const unsigned long long v = std::strtoull(t.c_str(), &e, 10);
    if (errno || *e != '\0' || t[0] == '-')
        throw std::invalid_argument("scan failed: '" + t + "' is not an index");
    return v;
}

double parse_value(const std::string& t) {
    if (t.empty())
        throw std::invalid_argument("scan failed");
    char* e = nullptr;
    const double v = std::strtod(t.c_str(), &e);
    if (*e != '\0')
        throw std::invalid_argument("scan failed: '" + t + "' is not a number");
    return v;
}

csr_host load_as_csr(const char* path) {
    mapped f(path);
    scanner sc(f.begin(), f.end());
    // banner (mm_read_banner): %%MatrixMarket matrix <format> <field> <symmetry>
    const std::string banner = sc.line();
    if (banner.rfind("%%MatrixMarket", 0) != 0)
        throw std::invalid_argument("not a Matrix Market file (missing %%MatrixMarket banner)");
    scanner bs(banner.data(), banner.data() + banner.size());
    bs.token();
    const std::string obj = lower(bs.token()), fmt = lower(bs.token()), field = lower(bs.token()),
                      symm = lower(bs.token());
    if (symm.empty())
        throw std::invalid_argument("malformed Matrix Market banner");
    if (obj != "matrix")
        throw std::invalid_argument("unsupported Matrix Market object '" + obj + "'");
    if (fmt != "coordinate")
        throw std::invalid_argument("Only coordinate matrix loading is implemented.");
    if (field == "complex")
        throw std::invalid_argument("complex Matrix Market matrices are not supported");
    const bool pattern = field == "pattern";
    const bool symmetric = symm == "symmetric" || symm == "hermitian";
    // comments and blank lines, then the size line
    std::string size_line;
    for (;;) {
        if (sc.at_end())
            throw std::invalid_argument("Matrix Market file has no size line");
        size_line = sc.line();
        const size_t first = size_line.find_first_not_of(" \t");
        if (first == std::string::npos || size_line[first] == '%')
            continue;
        break;
    }
    scanner ss(size_line.data(), size_line.data() + size_line.size());
    const uint64_t rows = parse_index(ss.token()), cols = parse_index(ss.token()), nnz = parse_index(ss.token());
    if (rows > 0xFFFFFFFFull || cols > 0xFFFFFFFFull)
        throw std::invalid_argument("matrix dimensions must fit in 32 bits");
    if (symmetric && rows != cols)  // each entry's mirror (col, row) must be a row of the matrix
        throw std::invalid_argument("a symmetric or Hermitian matrix must be square");
    // the size line sizes the allocations below: an entry takes at least four bytes ("1 1\n"), and the row
    // arrays must fit in the host's memory
    if (nnz > f.size() / 4)
        throw std::invalid_argument("the size line claims more entries than the file holds");
    const long pages = sysconf(_SC_PHYS_PAGES), page = sysconf(_SC_PAGE_SIZE);
    if (pages > 0 && page > 0 && (rows + 1) * 12 > (uint64_t)pages * (uint64_t)page)
        throw std::invalid_argument("the row count does not fit in the host's memory");
    // entries, in file order
    std::vector<uint32_t> r(nnz), c(nnz);
    std::vector<double> v(nnz, 1.0);
    for (uint64_t i = 0; i < nnz; ++i) {
        const uint64_t ri = parse_index(sc.token()), ci = parse_index(sc.token());
        if (!pattern)
            v[i] = parse_value(sc.token());
        if (ri < 1 || ci < 1 || ri > rows || ci > cols)
            throw std::invalid_argument("Matrix Market entry out of range");
        r[i] = (uint32_t)(ri - 1);
        c[i] = (uint32_t)(ci - 1);
    }
    // csr::from_coo over coo::iterate (each off-diagonal entry of a symmetric file, then its mirror)
    csr_host m;
    m.rows = (uint32_t)rows;
    m.cols = (uint32_t)cols;
    std::vector<uint64_t> count(rows + 1, 0);
    uint64_t total = 0;
    for (uint64_t i = 0; i < nnz; ++i) {
        ++count[r[i]];
        ++total;
        if (symmetric && r[i] != c[i]) {
            ++count[c[i]];
            ++total;
        }
    }
    if (total > 0xFFFFFFFFull)
        throw std::invalid_argument("too many non-zeros for 32-bit row offsets");
    m.row_ptr.assign(rows + 1, 0);
    for (uint64_t i = 0; i < rows; ++i)
        m.row_ptr[i + 1] = m.row_ptr[i] + (uint32_t)count[i];
    m.col.resize(total);
    m.val.resize(total);
    std::vector<uint32_t> next(m.row_ptr.begin(), m.row_ptr.end() - 1);
    auto put = [&](uint32_t row, uint32_t col, double val) {
        const uint32_t at = next[row]++;
        m.col[at] = col;
        m.val[at] = val;
    };
    for (uint64_t i = 0; i < nnz; ++i) {
        put(r[i], c[i], v[i]);
        if (symmetric && r[i] != c[i])
            put(c[i], r[i], v[i]);
    }
    std::vector<uint32_t> perm;
    std::vector<uint32_t> tc;
    std::vector<double> tv;
    for (uint64_t i = 0; i < rows; ++i) {
        const uint32_t b = m.row_ptr[i], e = m.row_ptr[i + 1];
        if (e - b < 2 || std::is_sorted(m.col.begin() + b, m.col.begin() + e))
            continue;
        perm.resize(e - b);
        std::iota(perm.begin(), perm.end(), 0u);
        std::stable_sort(perm.begin(), perm.end(), [&](uint32_t x, uint32_t y) { return m.col[b + x] < m.col[b + y]; });
        tc.resize(e - b);
        tv.resize(e - b);
        for (uint32_t k = 0; k < e - b; ++k) {
            tc[k] = m.col[b + perm[k]];
            tv[k] = m.val[b + perm[k]];
        }
        std::copy(tc.begin(), tc.end(), m.col.begin() + b);
        std::copy(tv.begin(), tv.end(), m.val.begin() + b);
    }
    return m;
}

template <typename F>
int guarded(const char* what, F&& f) {
    try {
        return f();
    } catch (const std::invalid_argument& e) {
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "%s: %s", what, e.what());
    } catch (const io_error& e) {
        return fail(DIMGPU_ERR_IO, "%s: %s", what, e.what());
    } catch (const std::bad_alloc&) {
        return fail(DIMGPU_ERR_OUT_OF_MEMORY, "%s: out of host memory", what);
    } catch (const std::exception& e) {
        return fail(DIMGPU_ERR_IO, "%s: %s", what, e.what());
    }
}

}  // namespace
}  // namespace mm
}  // namespace dimgpu

extern "C" {

int dimgpu_mm_csr_dimensions(const char* path, uint32_t* rows, uint32_t* cols, uint64_t* nnz) {
    using namespace dimgpu;
    if (!path || !*path || !rows || !cols || !nnz)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "NULL argument");
    return mm::guarded("load_as_csr", [&] {
        const mm::csr_host m = mm::load_as_csr(path);
        *rows = m.rows;
        *cols = m.cols;
        *nnz = m.col.size();
        return DIMGPU_OK;
    });
}

int dimgpu_mm_read_csr(const char* path, uint32_t* row_ptr, uint32_t* col_indices, double* values) {
    using namespace dimgpu;
    if (!path || !*path || !row_ptr)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "NULL argument");
    return mm::guarded("load_as_csr", [&] {
        const mm::csr_host m = mm::load_as_csr(path);
        if (!m.col.empty() && (!col_indices || !values))
            throw std::invalid_argument("NULL col_indices or values for a matrix with entries");
        std::copy(m.row_ptr.begin(), m.row_ptr.end(), row_ptr);
        std::copy(m.col.begin(), m.col.end(), col_indices);
        std::copy(m.val.begin(), m.val.end(), values);
        return DIMGPU_OK;
    });
}

}  // extern "C"
