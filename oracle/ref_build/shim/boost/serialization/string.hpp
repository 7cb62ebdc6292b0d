// Stand-in for a Boost header the reference's sources include; the compiled reference
// functions use nothing from it (it only serves serialisation and timing statistics).
#pragma once
