// Minimal stand-in for the parts of AMReX that the reference's per-cell
// numerics (Source/Src_3d/*.H) and per-case plugin headers (species.H,
// thermo.H, transport.H, userfuncs.H, chemistry.H and their .cpp files) use,
// so that those files compile unmodified on the host.  Test infrastructure
// only: it lets oracle/ref_driver.cpp call the reference's own compute_flux,
// update_residual, update_cutcells and compute_spec_source as the checker
// of the oracle restatement.
//
// Semantics follow AMReX's public interface:
//   Array4<T>      data pointer, j/k/n strides, begin/end (exclusive), ncomp;
//                  a(i,j,k,n) = p[(i-begin.x) + (j-begin.y) jstride
//                                 + (k-begin.z) kstride + n nstride]
//   GpuArray<T,N>  fixed-size array with operator[]
//   IntVect        three ints with operator[]
//   Math::abs      std::abs;  min, max: std::min, std::max
//   Gpu::ManagedVector  std::vector with dataPtr()
//   Abort          throws amrex_shim_abort (the driver turns it into a status)
//   Print          discards its output
//   ParmParse      queries leave their arguments unchanged (no inputs file)
// With MFG_COUNT_FLOPS defined, Real is a counting double (count_double.H):
// the same sources then report how many FP64 operations they perform.
#ifndef MFG_AMREX_SHIM_H_
#define MFG_AMREX_SHIM_H_

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#define AMREX_SPACEDIM 3
#define BL_SPACEDIM 3
#define AMREX_GPU_DEVICE
#define AMREX_GPU_HOST
#define AMREX_GPU_HOST_DEVICE
#define AMREX_GPU_DEVICE_MANAGED
#define AMREX_FORCE_INLINE inline
#define AMREX_INLINE inline
#define AMREX_RESTRICT __restrict__
#define AMREX_PRAGMA_SIMD
#define AMREX_D_DECL(a, b, c) a, b, c

#ifdef MFG_COUNT_FLOPS
#include "count_double.H"
#endif

namespace amrex {

#ifdef MFG_COUNT_FLOPS
using Real = mfg_count::CD;
#else
using Real = double;
#endif

template <class T>
using Vector = std::vector<T>;

struct Dim3 {
    int x, y, z;
};

struct IntVect {
    int v[3];
    IntVect() : v{0, 0, 0} {}
    IntVect(int i, int j, int k) : v{i, j, k} {}
    int& operator[](int d) { return v[d]; }
    const int& operator[](int d) const { return v[d]; }
};

template <class T, int N>
struct GpuArray {
    T arr[N];
    T& operator[](int i) { return arr[i]; }
    const T& operator[](int i) const { return arr[i]; }
};

template <class T>
struct Array4 {
    T* p = nullptr;
    int64_t jstride = 0, kstride = 0, nstride = 0;
    Dim3 begin{0, 0, 0}, end{0, 0, 0};
    int ncomp = 0;
    T& operator()(int i, int j, int k) const {
        return p[(int64_t)(i - begin.x) + (int64_t)(j - begin.y) * jstride + (int64_t)(k - begin.z) * kstride];
    }
    T& operator()(int i, int j, int k, int n) const {
        return p[(int64_t)(i - begin.x) + (int64_t)(j - begin.y) * jstride + (int64_t)(k - begin.z) * kstride +
                 (int64_t)n * nstride];
    }
    T& operator()(const IntVect& iv, int n) const { return (*this)(iv[0], iv[1], iv[2], n); }
};

// amrex::min / amrex::max (AMReX_Algorithm.H), reached unqualified through
// "using namespace amrex" in flux_schemes.H
template <class T>
inline const T& min(const T& a, const T& b) {
    return std::min(a, b);
}
template <class T>
inline const T& max(const T& a, const T& b) {
    return std::max(a, b);
}

namespace Math {
template <class T>
inline T abs(T x) {
    return std::abs(x);
}
}  // namespace Math

struct amrex_shim_abort : std::runtime_error {
    explicit amrex_shim_abort(const std::string& m) : std::runtime_error(m) {}
};

[[noreturn]] inline void Abort(const std::string& msg = "") { throw amrex_shim_abort(msg); }

struct Print {
    Print() {}
    template <class T>
    Print& operator<<(const T&) {
        return *this;
    }
};

struct ParmParse {
    explicit ParmParse(const std::string& = "") {}
    template <class T>
    int query(const char*, T&) const {
        return 0;
    }
    template <class T>
    void get(const char*, T&) const {}
    template <class T>
    int queryarr(const char*, std::vector<T>&) const {
        return 0;
    }
    template <class T>
    void getarr(const char*, std::vector<T>&) const {}
    int countval(const char*) const { return 0; }
    bool contains(const char*) const { return false; }
};

namespace Gpu {
template <class T>
struct ManagedVector : std::vector<T> {
    using std::vector<T>::vector;
    T* dataPtr() { return this->data(); }
    const T* dataPtr() const { return this->data(); }
};
}

}  // namespace amrex

#endif
