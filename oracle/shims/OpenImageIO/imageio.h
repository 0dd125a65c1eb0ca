// Shim: OpenImageIO is not available.  The oracle build never compiles the
// reference's Image.cpp / ImageFileLoader.cpp; image loading goes through
// oracle/shims/ref_support.cpp (PFM reader).
#pragma once
