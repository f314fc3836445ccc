/* Header-only GSL stand-in for compiling the reference KDTree sources as an oracle: nothing from this header is used on the KDTree path. */
#pragma once
