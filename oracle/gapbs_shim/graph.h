// Stand-in: the ParHDE sources include this gapbs header but use nothing from it.
#ifndef ORACLE_SHIM_GRAPH_H_
#define ORACLE_SHIM_GRAPH_H_
#include <cstdint>
#endif
