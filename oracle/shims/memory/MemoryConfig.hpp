// Stand-in for the configure-generated memory/MemoryConfig.hpp.
#pragma once
#define TOTAL_PHYSICAL_MEMORY 0
#define CACHE_LINE_SIZE 64
#define HAVE_POSIX_MEMALIGN
