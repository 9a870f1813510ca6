// Stand-in: logging is not used by the hot-path headers.
#pragma once
