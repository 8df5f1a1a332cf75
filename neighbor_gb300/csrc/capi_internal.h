// Shared pieces of the C ABI's translation units: handle types and status helpers.
#ifndef NEIGHBOR_GB300_CAPI_INTERNAL_H_
#define NEIGHBOR_GB300_CAPI_INTERNAL_H_

#include <exception>
#include <new>
#include <string>

#include <cuda_runtime.h>

#include "neighbor/neighbor.h"
#include "neighbor_gb300.h"

struct nbr_lbvh_s
    {
    neighbor::LBVH lbvh;
    };

struct nbr_traverser_s
    {
    neighbor::LBVHTraverser trav;
    };

namespace neighbor_capi
{
// The calling thread's last error message (defined in capi.cu).
void set_last_error(const std::string& msg);

inline int fail(int code, const std::string& msg)
    {
    set_last_error(msg);
    return code;
    }

// Map an exception from the C++ layer to a status code.
inline int from_exception(const std::exception& e)
    {
    const std::string m = e.what();
    if (m.find("allocating") != std::string::npos) return fail(NBR_ERR_ALLOC, m);
    if (m.find("bounded device wait") != std::string::npos) return fail(NBR_ERR_DEVICE_WAIT, m);
    if (m.find("Invalid") != std::string::npos || m.find("maximum of 32") != std::string::npos
        || m.find("must be") != std::string::npos || m.find("need") != std::string::npos)
        return fail(NBR_ERR_INVALID, m);
    return fail(NBR_ERR_CUDA, m);
    }

template<class F>
int guarded(F&& f)
    {
    try
        {
        f();
        set_last_error("");
        return NBR_OK;
        }
    catch (const std::bad_alloc&)
        {
        return fail(NBR_ERR_ALLOC, "host allocation failed");
        }
    catch (const std::exception& e)
        {
        return from_exception(e);
        }
    catch (...)
        {
        return fail(NBR_ERR_CUDA, "unknown error");
        }
    }

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }
inline float3 f3(const float v[3]) { return make_float3(v[0], v[1], v[2]); }
inline bool valid_block(unsigned int bs) { return bs >= 32 && bs <= 1024 && bs % 32 == 0; }
} // namespace neighbor_capi

#endif // NEIGHBOR_GB300_CAPI_INTERNAL_H_
