// Range-for stand-in for BOOST_FOREACH.
#pragma once
#define BOOST_FOREACH(decl, range) for (decl : range)
