// Stand-in for boost/program_options.hpp: Params declares (but the compiled functions
// never call) its command-line parsing.
#pragma once
namespace boost { namespace program_options {
class options_description {};
class variables_map {};
} }
