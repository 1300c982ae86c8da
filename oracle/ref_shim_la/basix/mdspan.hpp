// Stand-in for <basix/mdspan.hpp> (Basix is absent here): the reference
// names its mdspan namespace through MDSPAN_IMPL_STANDARD_NAMESPACE, and
// CCCL ships an implementation in cuda::std.
#pragma once
#include <cuda/std/mdspan>
#define MDSPAN_IMPL_STANDARD_NAMESPACE cuda::std
