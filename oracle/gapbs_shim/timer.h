// Stand-in: the ParHDE sources include this gapbs header but use nothing from it.
#ifndef ORACLE_SHIM_TIMER_H_
#define ORACLE_SHIM_TIMER_H_
#endif
