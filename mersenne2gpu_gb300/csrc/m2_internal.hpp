// m2_internal.hpp -- what one part of libm2gpu reads from a context that the
// C ABI does not expose: its digit layout, creation options, stream and
// device-side state.  Every call is stream-ordered on the context's stream.
#pragma once
#include "../../include/m2gpu.h"
#include "m2_host.hpp"

#include <cuda_runtime_api.h>

namespace m2k { struct LargePlan; }

namespace m2i {

// plan of the three-pass path for exponent layout L (false: no plan fits);
// carry_pairs is the -B hint (columns per CTA), 0 for the default
bool plan_large(const m2::Layout& L, int span, uint32_t carry_pairs, m2k::LargePlan& P);

// digit widths and bit positions of the context's residue
const m2::Layout& layout(const m2_ctx* c);
// the options of m2_create (device, hints, path, fields), with the stream
// cleared: a second context built from them has the same transform
m2_opts creation_opts(const m2_ctx* c);
cudaStream_t stream(const m2_ctx* c);

// the state's n canonical digits, written into the context's canonical
// buffer (device memory, valid until the context's next call)
int canonical(m2_ctx* c, const unsigned long long** out);
// the state's n signed digit words (device memory) for a caller that writes
// a new state there and reads it back through canonical(); pending segment
// carries are cleared
int raw_state(m2_ctx* c, long long** digits);
// the context's canonical buffer (device memory, n words), allocated if needed
int canon_buffer(m2_ctx* c, unsigned long long** buf);
// state <- the canonical digits in the canonical buffer (balanced on the
// device), with the iteration counter set
int load_canon(m2_ctx* c, uint32_t iteration);

}  // namespace m2i
