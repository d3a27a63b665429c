// lbffs_cl_compat.hpp -- the two OpenCL C++ names LBFFS's output fragment uses, mapped
// onto the C ABI, so D3Q19_opencl/write.hpp and D3Q27_opencl/write.hpp compile unchanged
// against a context.  write.hpp only ever calls
//     cl::copy(queue, X_d, X.begin(), X.end());          (write.hpp:3-14)
// i.e. a device -> host download of one whole buffer.
#ifndef LBFFS_CL_COMPAT_HPP
#define LBFFS_CL_COMPAT_HPP

#include <cstdio>
#include <cstdlib>
#include <iterator>

#include "lbffs_cuda.h"

namespace cl {

// stands in for cl::CommandQueue: the context the downloads go through
struct CommandQueue {
    lbffs_ctx* ctx;
};

// stands in for cl::Buffer: which device field of the context
struct Buffer {
    int field;
};

template <class It>
inline void copy(CommandQueue& queue, const Buffer& buffer, It first, It last)
{
    const size_t n = static_cast<size_t>(std::distance(first, last));
    const int rc = lbffs_download(queue.ctx, buffer.field, &*first, n * sizeof(*first));
    if (rc != LBFFS_OK) {
        std::fprintf(stderr, "lbffs_download(field %d): %s\n", buffer.field, lbffs_last_error(queue.ctx));
        std::exit(EXIT_FAILURE);
    }
}

}  // namespace cl

#endif
