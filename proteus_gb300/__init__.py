"""GB300-native relational hot path (radix partitioning, hash join, hash
group-by) behind a C ABI; see include/gbjoin.h.  ``engine`` holds the
host-side Python wrapper over that ABI."""
