// handles.cuh — the opaque handle behind cp_mesh and the internal helpers the
// C-ABI translation units share.
#pragma once

#include <string>

#include "../../include/cpq.h"
#include "bvh.cuh"

struct cp_mesh {
    cpq::Bvh bvh;
};

namespace cpq {

// Validate cp_query_opts (NULL = defaults) into QueryParams; sets the error string.
cp_status parse_query_opts(const cp_query_opts* opts, QueryParams* out);

// Record `msg` as the calling thread's last error and return `s`.
cp_status set_error(cp_status s, const std::string& msg);

}  // namespace cpq
