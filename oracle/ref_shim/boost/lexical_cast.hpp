// Stand-in: the reference only names boost::lexical_cast in a using-declaration.
#pragma once
namespace boost {
template <class Target, class Source> Target lexical_cast(const Source &);
}
