// Minimal stand-in for the part of libtorch's C++ API that the reference's
// pyDeform sources use (torch::Tensor with size(), storage().data(),
// torch::full and TensorOptions().dtype()), so that those sources compile
// unchanged into oracle/_ref without libtorch or pybind11.  A Tensor is a
// contiguous row-major buffer, either owned (made by full) or a view of
// caller memory (made by torch::refshim::wrap in the C wrapper).
#ifndef MO_REFSHIM_TORCH_EXTENSION_
#define MO_REFSHIM_TORCH_EXTENSION_

#include <cstdint>
#include <cstring>
#include <initializer_list>
#include <memory>
#include <stdexcept>
#include <vector>

namespace torch {

enum ScalarType { kFloat32, kFloat64, kInt32, kInt64 };

inline size_t element_size(ScalarType t) { return (t == kFloat64 || t == kInt64) ? 8 : 4; }

struct TensorOptions {
    ScalarType dt = kFloat32;
    TensorOptions dtype(ScalarType t) const {
        TensorOptions o = *this;
        o.dt = t;
        return o;
    }
};

struct Storage {
    void* p;
    void* data() const { return p; }
};

class Tensor {
public:
    Tensor() = default;
    int64_t size(int64_t d) const {
        if (d < 0) d += (int64_t)sizes_.size();
        if (d < 0 || d >= (int64_t)sizes_.size()) throw std::out_of_range("Tensor::size: bad dimension");
        return sizes_[(size_t)d];
    }
    int64_t dim() const { return (int64_t)sizes_.size(); }
    int64_t numel() const {
        int64_t n = 1;
        for (int64_t s : sizes_) n *= s;
        return n;
    }
    ScalarType dtype() const { return dtype_; }
    Storage storage() const { return Storage{data_}; }

    static Tensor make(const std::vector<int64_t>& sizes, ScalarType t, void* external) {
        Tensor x;
        x.sizes_ = sizes;
        x.dtype_ = t;
        if (external) {
            x.data_ = external;
        } else {
            x.own_ = std::make_shared<std::vector<unsigned char>>((size_t)x.numel() * element_size(t));
            x.data_ = x.own_->data();
        }
        return x;
    }

private:
    std::shared_ptr<std::vector<unsigned char>> own_;
    void* data_ = nullptr;
    std::vector<int64_t> sizes_;
    ScalarType dtype_ = kFloat32;
};

inline Tensor full(std::initializer_list<int64_t> sizes, double value, TensorOptions o) {
    Tensor t = Tensor::make(std::vector<int64_t>(sizes), o.dt, nullptr);
    void* p = t.storage().data();
    const int64_t n = t.numel();
    for (int64_t i = 0; i < n; ++i) {
        switch (o.dt) {
            case kFloat32: static_cast<float*>(p)[i] = (float)value; break;
            case kFloat64: static_cast<double*>(p)[i] = value; break;
            case kInt32: static_cast<int32_t*>(p)[i] = (int32_t)value; break;
            case kInt64: static_cast<int64_t*>(p)[i] = (int64_t)value; break;
        }
    }
    return t;
}

namespace refshim {
// A view of caller memory with the given shape (no copy).
inline Tensor wrap(const void* p, std::initializer_list<int64_t> sizes, ScalarType t) {
    return Tensor::make(std::vector<int64_t>(sizes), t, const_cast<void*>(p));
}
}  // namespace refshim

}  // namespace torch

#endif
