// Runs the host file readers over every file of a directory: `driver <dir>` reads each file as an HDF5
// file (the CSR group "A" and the vector "Y"), `driver <dir> mm` as a Matrix Market file.  Built with
// AddressSanitizer and UBSan by tests/test_readers_sanitized.py, so that any out-of-bounds access or
// undefined behaviour on a corrupted file stops it with a report.
#include <dirent.h>

#include <algorithm>
#include <cstdio>
#include <string>
#include <vector>

#include "dimgpu.h"
int main(int argc, char** argv) {
    std::vector<std::string> names;
    if (argc < 2)
        return 2;
    DIR* d = opendir(argv[1]);
    if (!d)
        return 2;
    for (dirent* e; (e = readdir(d));)
        if (e->d_name[0] != '.')
            names.push_back(e->d_name);
    closedir(d);
    std::sort(names.begin(), names.end());
    const bool mm = argc > 2 && std::string(argv[2]) == "mm";
    long ok = 0, err = 0;
    for (const auto& n : names) {
        const std::string p = std::string(argv[1]) + "/" + n;
        uint32_t rows = 0, cols = 0;
        uint64_t nnz = 0, len = 0;
        int rc = mm ? dimgpu_mm_csr_dimensions(p.c_str(), &rows, &cols, &nnz)
                    : dimgpu_h5_csr_dimensions(p.c_str(), "A", &rows, &cols, &nnz);
        if (rc == 0 && rows < (1u << 24) && nnz < (1ull << 26)) {
            std::vector<uint32_t> rp(rows + 1), ci(nnz + 1);
            std::vector<double> v(nnz + 1);
            rc = mm ? dimgpu_mm_read_csr(p.c_str(), rp.data(), ci.data(), v.data())
                    : dimgpu_h5_read_matlab_compatible(p.c_str(), "A", rp.data(), ci.data(), v.data());
        }
        (rc == 0 ? ok : err)++;
        if (!mm) {
            rc = dimgpu_h5_vector_length(p.c_str(), "Y", &len);
            if (rc == 0 && len < (1ull << 26)) {
                std::vector<double> y(len + 1);
                rc = dimgpu_h5_read_vector(p.c_str(), "Y", y.data());
            }
            (rc == 0 ? ok : err)++;
        }
    }
    printf("files %zu ok %ld err %ld\n", names.size(), ok, err);
    return 0;
}
