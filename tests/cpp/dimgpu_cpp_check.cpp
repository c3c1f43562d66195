// A C++ caller of dimgpu through include/dimgpu.hpp, as a dim user would write it: from_csr, spmv on
// host spans and on device memory (CUDA runtime allocations, a stream, the status query), the CG
// solver, the SpMM, block CG and adjoint solve, the reference's exceptions, and the file IO (HDF5: write_matlab_compatible and
// read_matlab_compatible, store and load_csr5, the result vector; Matrix Market: load_matrix_market).
//
//   dimgpu_cpp_check <output file>
//
// Builds the 2-D 5-point Laplacian on a 64 x 64 grid, multiplies x_i = sin(0.37 i), solves A z = A x,
// and writes n, x, y = A x and z (little-endian doubles after a u64 n) for the test to compare with the
// oracle.  With DIMGPU_WITH_REFERENCE_CSR the matrix is the reference's own dim::mat::csr<double>
// (include/dim/mat/storage_formats/csr.h); otherwise a struct with the same members stands in for it.
#include <dimgpu.hpp>

#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <type_traits>
#include <vector>

#ifdef DIMGPU_WITH_REFERENCE_CSR
#include <dim/mat/storage_formats/csr.h>
using csr_t = dim::mat::csr<double>;
static csr_t make_csr(uint32_t n, const std::vector<double>& v, const std::vector<uint32_t>& rp,
                      const std::vector<uint32_t>& ci) {
    return csr_t{dim::mat::dimensions_t{.rows = n, .cols = n}, csr_t::values_t(v.begin(), v.end()),
                 csr_t::indices_t(rp.begin(), rp.end()), csr_t::indices_t(ci.begin(), ci.end())};
}
#else
struct csr_t {
    struct {
        uint32_t rows, cols;
    } dimensions;
    std::vector<double> values;
    std::vector<uint32_t> row_start_offsets;
    std::vector<uint32_t> col_indices;
};
static csr_t make_csr(uint32_t n, const std::vector<double>& v, const std::vector<uint32_t>& rp,
                      const std::vector<uint32_t>& ci) {
    return csr_t{{n, n}, v, rp, ci};
}
#endif

static_assert(!std::is_copy_constructible_v<dim::gpu::csr5> && !std::is_copy_assignable_v<dim::gpu::csr5>);
static_assert(std::is_nothrow_move_constructible_v<dim::gpu::csr5> && std::is_nothrow_move_assignable_v<dim::gpu::csr5>);
static_assert(!std::is_copy_constructible_v<dim::gpu::calibrator> && !std::is_copy_constructible_v<dim::gpu::cg_solver>);

#define EXPECT(c)                                                        \
    do {                                                                 \
        if (!(c)) {                                                      \
            std::fprintf(stderr, "%s:%d: failed: %s\n", __FILE__, __LINE__, #c); \
            return 1;                                                    \
        }                                                                \
    } while (0)

int main(int argc, char** argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s <output file>\n", argv[0]);
        return 2;
    }
    const uint32_t g = 64, n = g * g;
    std::vector<double> v;
    std::vector<uint32_t> rp{0}, ci;
    for (uint32_t i = 0; i < g; ++i)
        for (uint32_t j = 0; j < g; ++j) {
            const uint32_t r = i * g + j;
            if (i > 0) ci.push_back(r - g), v.push_back(-1.0);
            if (j > 0) ci.push_back(r - 1), v.push_back(-1.0);
            ci.push_back(r), v.push_back(4.0);
            if (j + 1 < g) ci.push_back(r + 1), v.push_back(-1.0);
            if (i + 1 < g) ci.push_back(r + g), v.push_back(-1.0);
            rp.push_back((uint32_t)ci.size());
        }
    const csr_t m = make_csr(n, v, rp, ci);

    dim::gpu::csr5 tmp = dim::gpu::csr5::from_csr(m);
    dim::gpu::csr5 A = std::move(tmp);  // move-only handle; tmp is empty now
    EXPECT(tmp.handle() == nullptr && A.handle() != nullptr);
    EXPECT(A.non_zero_count() == v.size() && A.dimensions().rows == n);

    std::vector<double> x(n), y(n), z(n, 0.0);
    for (uint32_t i = 0; i < n; ++i)
        x[i] = std::sin(0.37 * i);
    A.spmv(x, y);

    // the reference's exception on a size mismatch (csr5.h:820-821)
    bool threw = false;
    try {
        std::vector<double> short_x(n - 1);
        A.spmv(short_x, y);
    } catch (const std::invalid_argument&) {
        threw = true;
    }
    EXPECT(threw);

    // the same product on device memory with a calibrator, asynchronous on a stream
    dim::gpu::calibrator cal = A.create_calibrator();
    EXPECT(cal.handle() != nullptr);
    double *dx = nullptr, *dy = nullptr;
    EXPECT(cudaMalloc(&dx, n * sizeof(double)) == cudaSuccess && cudaMalloc(&dy, n * sizeof(double)) == cudaSuccess);
    cudaStream_t s = nullptr;
    EXPECT(cudaStreamCreate(&s) == cudaSuccess);
    EXPECT(cudaMemcpyAsync(dx, x.data(), n * sizeof(double), cudaMemcpyHostToDevice, s) == cudaSuccess);
    A.spmv_device(dx, dy, &cal, s);
    A.status(&cal, s);  // synchronizes; throws if the product recorded a failure
    std::vector<double> y_dev(n);
    EXPECT(cudaMemcpy(y_dev.data(), dy, n * sizeof(double), cudaMemcpyDeviceToHost) == cudaSuccess);
    EXPECT(y_dev == y);  // the same kernel on the same input: the same bits
    cudaFree(dx);
    cudaFree(dy);
    cudaStreamDestroy(s);

    dimgpu_cg_params p{};
    p.tol = 1e-10;
    p.max_it = 10000;
    p.precision = DIMGPU_CG_FP64;
    p.use_graph = 1;
    dim::gpu::cg_solver solver(A, p);
    const dimgpu_cg_stats st = solver.solve(y, z);
    EXPECT(st.status == DIMGPU_OK && st.rel_residual <= 1.5e-10);
    A.status();

    // the batched and differentiated forms: an SpMM with two copies of x, a block CG on [y, 2 y], and the
    // adjoint solve of A lambda = y (A is symmetric); all on device memory
    {
        std::vector<double> X2(2 * n), Y2(2 * n), B2(2 * n), Z2(2 * n, 0.0);
        for (uint32_t i = 0; i < n; ++i) {
            X2[2 * i] = X2[2 * i + 1] = x[i];
            B2[2 * i] = y[i];
            B2[2 * i + 1] = 2.0 * y[i];
        }
        double *dX2 = nullptr, *dY2 = nullptr, *dB2 = nullptr, *dZ2 = nullptr, *dl = nullptr, *dg = nullptr;
        EXPECT(cudaMalloc(&dX2, 2 * n * sizeof(double)) == cudaSuccess && cudaMalloc(&dY2, 2 * n * sizeof(double)) == cudaSuccess);
        EXPECT(cudaMalloc(&dB2, 2 * n * sizeof(double)) == cudaSuccess && cudaMalloc(&dZ2, 2 * n * sizeof(double)) == cudaSuccess);
        EXPECT(cudaMalloc(&dl, n * sizeof(double)) == cudaSuccess && cudaMalloc(&dg, n * sizeof(double)) == cudaSuccess);
        EXPECT(cudaMemcpy(dX2, X2.data(), 2 * n * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess);
        A.spmm_device(2, dX2, 2, dY2, 2);
        EXPECT(cudaMemcpy(Y2.data(), dY2, 2 * n * sizeof(double), cudaMemcpyDeviceToHost) == cudaSuccess);
        for (uint32_t i = 0; i < n; ++i)
            EXPECT(std::fabs(Y2[2 * i] - y[i]) <= 1e-12 * 8.0 && Y2[2 * i + 1] == Y2[2 * i]);
        EXPECT(cudaMemcpy(dB2, B2.data(), 2 * n * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess);
        EXPECT(cudaMemcpy(dZ2, Z2.data(), 2 * n * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess);
        dim::gpu::block_cg_solver bcg(A, 2, p);
        std::vector<int64_t> its(2);
        std::vector<double> rel(2);
        const dimgpu_block_cg_stats bst = bcg.solve_device(dB2, 2, dZ2, 2, its, rel);
        EXPECT(bst.converged_columns == 2 && rel[0] <= 1.5e-10 && rel[1] <= 1.5e-10);
        EXPECT(cudaMemcpy(Z2.data(), dZ2, 2 * n * sizeof(double), cudaMemcpyDeviceToHost) == cudaSuccess);
        for (uint32_t i = 0; i < n; ++i)  // A z = A x: the solutions are x and 2 x
            EXPECT(std::fabs(Z2[2 * i] - x[i]) <= 1e-6 && std::fabs(Z2[2 * i + 1] - 2.0 * x[i]) <= 2e-6);
        // adjoint: lambda = A^{-T} y = x (A symmetric, y = A x), dL/dA on the pattern = -lambda x^T
        std::vector<double> zero(n, 0.0), grad(v.size());
        double* dgrad = nullptr;
        EXPECT(cudaMalloc(&dgrad, v.size() * sizeof(double)) == cudaSuccess);
        EXPECT(cudaMemcpy(dg, y.data(), n * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess);
        EXPECT(cudaMemcpy(dl, zero.data(), n * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess);
        EXPECT(cudaMemcpy(dX2, x.data(), n * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess);
        const dimgpu_cg_stats ast = dim::gpu::cg_adjoint(A, dg, dX2, dl, dgrad, p);
        EXPECT(ast.status == DIMGPU_OK);
        std::vector<double> lam(n);
        EXPECT(cudaMemcpy(lam.data(), dl, n * sizeof(double), cudaMemcpyDeviceToHost) == cudaSuccess);
        EXPECT(cudaMemcpy(grad.data(), dgrad, v.size() * sizeof(double), cudaMemcpyDeviceToHost) == cudaSuccess);
        for (uint32_t i = 0; i < n; ++i) {
            EXPECT(std::fabs(lam[i] - x[i]) <= 1e-6);
            for (uint32_t e = rp[i]; e < rp[i + 1]; ++e)
                EXPECT(grad[e] == -lam[i] * x[ci[e]]);
        }
        for (double* q : {dX2, dY2, dB2, dZ2, dl, dg, dgrad})
            cudaFree(q);
    }

    // HDF5 round trips next to the output file: the matrix through its MATLAB-compatible group and its
    // CSR5 group (converted with the reference's layout), the solution as a result vector
    const std::string h5path = std::string(argv[1]) + ".h5";
    dim::gpu::io::write_matlab_compatible(h5path, "A", m);
    const dim::gpu::io::csr_matrix back = dim::gpu::io::read_matlab_compatible(h5path, "A");
    EXPECT(back.dimensions.rows == n && back.values == v && back.row_start_offsets == rp && back.col_indices == ci);
    dimgpu_csr5_options ref_layout{16, 4, DIMGPU_LAYOUT_REFERENCE, 0};
    const dim::gpu::csr5 R = dim::gpu::csr5::from_csr(back, &ref_layout);
    dim::gpu::io::store(h5path, "A5", R, /*append=*/true);
    const dim::gpu::csr5 L = dim::gpu::io::load_csr5(h5path, "A5");
    std::vector<double> y5(n);
    L.spmv(x, y5);
    EXPECT(y5 == y);  // the same matrix, the same kernel: the same bits
    // the same matrix through a Matrix Market file (written here, general coordinate form)
    const std::string mtxpath = std::string(argv[1]) + ".mtx";
    FILE* mf = std::fopen(mtxpath.c_str(), "w");
    EXPECT(mf != nullptr);
    std::fprintf(mf, "%%%%MatrixMarket matrix coordinate real general\n%% written by the check\n%u %u %zu\n", n, n,
                 v.size());
    for (uint32_t r = 0; r < n; ++r)
        for (uint32_t e = rp[r]; e < rp[r + 1]; ++e)
            std::fprintf(mf, "%u %u %.17g\n", r + 1, ci[e] + 1, v[e]);
    std::fclose(mf);
    const dim::gpu::io::csr_matrix mmx = dim::gpu::io::load_matrix_market(mtxpath);
    EXPECT(mmx.values == v && mmx.row_start_offsets == rp && mmx.col_indices == ci);
    dim::gpu::io::write_vector(h5path, "z", z);
    EXPECT(dim::gpu::io::read_vector(h5path, "z") == z);
    threw = false;
    try {
        (void)dim::gpu::io::read_matlab_compatible(h5path, "missing");
    } catch (const std::invalid_argument&) {
        threw = true;
    }
    EXPECT(threw);

    FILE* f = std::fopen(argv[1], "wb");
    EXPECT(f != nullptr);
    const uint64_t nn = n;
    std::fwrite(&nn, sizeof(nn), 1, f);
    std::fwrite(x.data(), sizeof(double), n, f);
    std::fwrite(y.data(), sizeof(double), n, f);
    std::fwrite(z.data(), sizeof(double), n, f);
    std::fclose(f);
    std::printf("ok %lld iterations\n", (long long)st.iterations);
    return 0;
}
