// TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT (ds_compat; see core/Globals.h).
//
// An intrusively reference-counted base (SharedObject) and its smart pointer
// (Reference<T>): the object is deleted when the last Reference to it goes.
#pragma once

#include <atomic>
#include <cstdint>
#include <utility>
#include "Globals.h"

namespace cg
{

class SharedObject
{
public:
    SharedObject() = default;
    SharedObject(const SharedObject&) {}
    SharedObject& operator=(const SharedObject&) { return *this; }
    virtual ~SharedObject() = default;

    void acquire() const { _refs.fetch_add(1, std::memory_order_relaxed); }
    void release() const
    {
        if (_refs.fetch_sub(1, std::memory_order_acq_rel) == 1) delete this;
    }
    uint32_t referenceCount() const { return _refs.load(); }

private:
    mutable std::atomic<uint32_t> _refs {0};
};

template<typename T>
class Reference
{
public:
    Reference() = default;
    Reference(T* p) : _p{p} { if (_p) _p->acquire(); }
    Reference(const Reference& r) : _p{r._p} { if (_p) _p->acquire(); }
    Reference(Reference&& r) noexcept : _p{r._p} { r._p = nullptr; }
    template<typename U> Reference(const Reference<U>& r) : _p{r.get()} { if (_p) _p->acquire(); }
    ~Reference() { if (_p) _p->release(); }

    Reference& operator=(const Reference& r) { Reference t(r); std::swap(_p, t._p); return *this; }
    Reference& operator=(Reference&& r) noexcept { std::swap(_p, r._p); return *this; }
    Reference& operator=(T* p) { Reference t(p); std::swap(_p, t._p); return *this; }

    T* get() const { return _p; }
    T* operator->() const { return _p; }
    T& operator*() const { return *_p; }
    explicit operator bool() const { return _p != nullptr; }
    operator T*() const { return _p; }

private:
    T* _p = nullptr;
};

template<typename T, typename... Args>
Reference<T> makeUse(Args&&... args) { return Reference<T>(new T(std::forward<Args>(args)...)); }

} // namespace cg
