// Project-written stand-in for the reference's missing Copy.h, which is
// included by RadixSortLSD.h:35, RadixSelect.h:29 and RadixPartition.h:27 but
// is not in the reference tree.  The only names the included code needs from
// it are memcpy (<cstring>) and the `byte` type used by RadixSelect.h:74,77.
#pragma once
#include <cstring>
typedef unsigned char byte;
