// Reference-counted CUDA arrays.
//
// shared_array<T> and buffered_array<T> keep the reference's interface
// (include/neighbor/Memory.h:29-296): shared ownership through copies, get(), size(), host-side
// operator[] (the storage is CUDA managed memory, so results can be read on the host after a
// synchronize), a std::runtime_error when allocation fails, and a double buffer whose flip()
// swaps which half is current.
//
// device_array<T> is new: plain device memory for internal buffers that the host never indexes
// (sort ping-pong buffers, scan state, compressed nodes).  It grows and never shrinks.
#ifndef NEIGHBOR_MEMORY_H_
#define NEIGHBOR_MEMORY_H_

#include <algorithm>
#include <atomic>
#include <cstddef>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>

#include <cuda_runtime.h>

namespace neighbor
{
namespace detail
{
// Fault injection for tests: the next n allocations of shared_array / device_array fail as if
// the CUDA allocator had refused them (set through nbr_debug_inject_alloc_failures).
inline std::atomic<unsigned int>& injected_alloc_failures()
    {
    static std::atomic<unsigned int> n(0u);
    return n;
    }
inline bool take_injected_alloc_failure()
    {
    std::atomic<unsigned int>& n = injected_alloc_failures();
    unsigned int v = n.load();
    while (v > 0u && !n.compare_exchange_weak(v, v - 1u)) {}
    return v > 0u;
    }
// cudaMalloc / cudaMallocManaged, or the injected failure
inline cudaError_t device_malloc(void** p, size_t bytes, bool managed)
    {
    if (take_injected_alloc_failure()) return cudaErrorMemoryAllocation;
    return managed ? cudaMallocManaged(p, bytes) : cudaMalloc(p, bytes);
    }
} // namespace detail

template<typename T>
class shared_array
    {
    public:
        shared_array() : size_(0) {}

        explicit shared_array(size_t count) : size_(0) { allocate(count); }

        shared_array(const shared_array& other) = default;
        shared_array& operator=(const shared_array& other) = default;

        shared_array(shared_array&& other) noexcept
            : data_(std::move(other.data_)), size_(other.size_)
            {
            other.size_ = 0;
            }

        shared_array& operator=(shared_array&& other) noexcept
            {
            if (this != &other)
                {
                data_ = std::move(other.data_);
                size_ = other.size_;
                other.size_ = 0;
                }
            return *this;
            }

        void swap(shared_array& other)
            {
            std::swap(data_, other.data_);
            std::swap(size_, other.size_);
            }

        T& operator[](size_t idx) { return data_.get()[idx]; }
        const T& operator[](size_t idx) const { return data_.get()[idx]; }

        T* get() { return data_.get(); }
        const T* get() const { return data_.get(); }

        size_t size() const { return size_; }

    private:
        std::shared_ptr<T> data_;
        size_t size_;

        struct deleter
            {
            void operator()(T* ptr) const
                {
                if (ptr) cudaFree(ptr);
                }
            };

        void allocate(size_t count)
            {
            if (count == 0)
                {
                data_.reset();
                size_ = 0;
                return;
                }
            T* ptr = nullptr;
            const cudaError_t code = detail::device_malloc(reinterpret_cast<void**>(&ptr), count * sizeof(T), true);
            if (code != cudaSuccess)
                {
                (void)cudaGetLastError();
                data_.reset();
                size_ = 0;
                throw std::runtime_error(std::string("Error allocating managed memory: ")
                                         + cudaGetErrorString(code));
                }
            data_ = std::shared_ptr<T>(ptr, deleter());
            size_ = count;
            }
    };

template<typename T>
class buffered_array
    {
    public:
        buffered_array() : selector_(0) {}
        explicit buffered_array(size_t count) : x_(count), y_(count), selector_(0) {}

        void swap(buffered_array& other)
            {
            x_.swap(other.x_);
            y_.swap(other.y_);
            std::swap(selector_, other.selector_);
            }

        shared_array<T>& current() { return selector_ == 0 ? x_ : y_; }
        const shared_array<T>& current() const { return selector_ == 0 ? x_ : y_; }
        shared_array<T>& alternate() { return selector_ == 0 ? y_ : x_; }
        const shared_array<T>& alternate() const { return selector_ == 0 ? y_ : x_; }

        void flip() { selector_ ^= 1; }

        size_t size() const { return x_.size(); }

    private:
        shared_array<T> x_;
        shared_array<T> y_;
        int selector_;
    };

// Device-only growable buffer.
template<typename T>
class device_array
    {
    public:
        device_array() : ptr_(nullptr), size_(0) {}
        ~device_array() { release(); }
        device_array(const device_array&) = delete;
        device_array& operator=(const device_array&) = delete;

        // Ensure room for count elements; contents are not preserved when it grows.
        void reserve(size_t count)
            {
            if (count <= size_) return;
            release();
            T* p = nullptr;
            const cudaError_t code = detail::device_malloc(reinterpret_cast<void**>(&p), count * sizeof(T), false);
            if (code != cudaSuccess)
                {
                (void)cudaGetLastError();
                throw std::runtime_error(std::string("Error allocating device memory: ")
                                         + cudaGetErrorString(code));
                }
            ptr_ = p;
            size_ = count;
            }

        // Ensure room for count elements keeping the first `keep` (copied on `stream`).
        void grow(size_t count, size_t keep, cudaStream_t stream)
            {
            if (count <= size_) return;
            T* p = nullptr;
            const cudaError_t code = detail::device_malloc(reinterpret_cast<void**>(&p), count * sizeof(T), false);
            if (code != cudaSuccess)
                {
                (void)cudaGetLastError();
                throw std::runtime_error(std::string("Error allocating device memory: ")
                                         + cudaGetErrorString(code));
                }
            if (ptr_ && keep)
                {
                const cudaError_t c2 = cudaMemcpyAsync(p, ptr_, std::min(keep, size_) * sizeof(T),
                                                       cudaMemcpyDeviceToDevice, stream);
                if (c2 == cudaSuccess) (void)cudaStreamSynchronize(stream);
                }
            release();
            ptr_ = p;
            size_ = count;
            }

        T* get() { return ptr_; }
        const T* get() const { return ptr_; }
        size_t size() const { return size_; }

    private:
        T* ptr_;
        size_t size_;
        void release()
            {
            if (ptr_) cudaFree(ptr_);
            ptr_ = nullptr;
            size_ = 0;
            }
    };

} // namespace neighbor

#endif // NEIGHBOR_MEMORY_H_
