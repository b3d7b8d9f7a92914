/* Test infrastructure (oracle build only); see ../filtering_stream.hpp. */
#pragma once
#include "../filtering_stream.hpp"
