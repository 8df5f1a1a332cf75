// One tunable launch parameter plus its valid set.
//
// Interface as in the reference (include/neighbor/Tunable.h:39-118): construct from a
// [begin, end] range with a step or from a list, getTunableParameters(), setTunableParameters(),
// LaunchParameters{tunable, stream}, and checkParameter() throwing std::runtime_error for a value
// outside the set.
#ifndef NEIGHBOR_TUNABLE_H_
#define NEIGHBOR_TUNABLE_H_

#include <set>
#include <stdexcept>
#include <vector>

#include <cuda_runtime.h>

namespace neighbor
{

template<typename T>
class Tunable
    {
    public:
        Tunable(T begin, T end, T step)
            {
            for (T v = begin; v <= end; v += step) m_params.insert(v);
            }

        explicit Tunable(const std::vector<T>& params) { setTunableParameters(params); }

        std::vector<T> getTunableParameters() const { return std::vector<T>(m_params.begin(), m_params.end()); }

        void setTunableParameters(const std::vector<T>& params) { m_params = std::set<T>(params.begin(), params.end()); }

        struct LaunchParameters
            {
            typedef T type;
            explicit LaunchParameters(T tunable_) : tunable(tunable_), stream(0) {}
            LaunchParameters(T tunable_, cudaStream_t stream_) : tunable(tunable_), stream(stream_) {}
            T tunable;
            cudaStream_t stream;
            };

        T checkParameter(const LaunchParameters& params) const
            {
            if (m_params.find(params.tunable) == m_params.end())
                throw std::runtime_error("Invalid tuning parameter.");
            return params.tunable;
            }

    private:
        std::set<T> m_params;
    };

} // namespace neighbor

#endif // NEIGHBOR_TUNABLE_H_
