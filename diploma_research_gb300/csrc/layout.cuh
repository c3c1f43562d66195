// layout.cuh -- the CSR5 data layout in HBM, for the reference layout and the 32-lane device layout.
//
// A CSR5 matrix here is the reference's csr5_info_t (include/dim/mat/storage_formats/csr5.h:287-447)
// built at a chosen (sigma, omega):
//
//   tile_ptr[T+1]        u32; first row of each tile, MSB set when the tile holds an empty row
//   tile_desc[T*omega]   one packed word per tile column: y_offset | scansum_offset | bit_flag,
//                        fields of bit_width(sigma*omega), bit_width(omega) and sigma bits, packed
//                        from the least significant bit like GCC lays out csr5.h:39-41; u32 when
//                        they fit in 32 bits, else u64
//   tdo_ptr[T+1], tdo[]  tile_desc_offset_ptr / tile_desc_offset: row of each segment of a tile
//                        that contains empty rows (csr5.h:342-397)
//   vals[nnz], col[nnz]  the CSR arrays with full tiles re-ordered so that a lane reads its column
//                        row by row
//
// Two element orders inside such a tile:
//   kLayoutReference: element (column c, row r) at r*omega + c            (csr5.h:463-493)
//   kLayoutDevice:    f64 values in pairs  (r/2)*2*omega + 2c + r%2 (one 16-byte load = 2 rows),
//                     u32 columns and f32 values in quads (r/4)*4*omega + 4c + r%4 (16 bytes = 4 rows)
// The reference order re-orders only tiles spanning more than one row (single-row "fast-track"
// tiles stay in CSR order, csr5.h:466-468); the device orders re-order every full tile, so that the
// pair reads of values and the quad reads of column indices always meet the same elements.  The
// tail (the last nnz mod sigma*omega elements) stays in CSR order.
#pragma once

#include <cstdint>

namespace dimgpu {

enum layout_kind : int { kLayoutReference = 0, kLayoutDevice = 1 };

constexpr uint32_t kDirty = 0x80000000u;

__host__ __device__ constexpr uint32_t bit_width_u64(uint64_t v) {
    uint32_t w = 0;
    while (v) {
        ++w;
        v >>= 1;
    }
    return w;
}

struct desc_fields {
    uint32_t yb, sb, fb;
    __host__ __device__ constexpr uint32_t total() const { return yb + sb + fb; }
};

__host__ __device__ constexpr desc_fields fields_for(uint32_t sigma, uint32_t omega) {
    return desc_fields{bit_width_u64(uint64_t(sigma) * omega), bit_width_u64(omega), sigma};
}

// Position of element (column c, row r) of a re-ordered tile.
__host__ __device__ inline uint32_t pos_reference(uint32_t c, uint32_t r, uint32_t omega) { return r * omega + c; }
__host__ __device__ inline uint32_t pos_device_f64(uint32_t c, uint32_t r, uint32_t omega) {
    return (r >> 1) * (2 * omega) + 2 * c + (r & 1);
}
__host__ __device__ inline uint32_t pos_device_q32(uint32_t c, uint32_t r, uint32_t omega) {
    return (r >> 2) * (4 * omega) + 4 * c + (r & 3);
}

}  // namespace dimgpu
