// NVTX ranges around the library's stages (build, traversals, one-pass lists, capacity
// prediction and training, batched runs), shown by Nsight tools.  Without an attached tool a
// range costs a function-pointer check; defining NEIGHBOR_NO_NVTX removes them.
#ifndef NEIGHBOR_TRACE_H_
#define NEIGHBOR_TRACE_H_

#ifndef NEIGHBOR_NO_NVTX
#include <nvtx3/nvToolsExt.h>
#endif

namespace neighbor
{
namespace detail
{
class TraceRange
    {
    public:
        explicit TraceRange(const char* name)
            {
#ifndef NEIGHBOR_NO_NVTX
            nvtxRangePushA(name);
#else
            (void)name;
#endif
            }
        ~TraceRange()
            {
#ifndef NEIGHBOR_NO_NVTX
            nvtxRangePop();
#endif
            }
        TraceRange(const TraceRange&) = delete;
        TraceRange& operator=(const TraceRange&) = delete;
    };
} // namespace detail
} // namespace neighbor

#endif // NEIGHBOR_TRACE_H_
