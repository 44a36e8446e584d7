/* Stand-in for Intel's ittnotify.h so the reference's root gppKer.cpp, which
 * brackets its timed loop with VTune markers, compiles without VTune. */
#ifndef FK_ITTNOTIFY_SHIM_H
#define FK_ITTNOTIFY_SHIM_H
#define __SSC_MARK(x) ((void)0)
static inline void __itt_resume(void) {}
static inline void __itt_pause(void) {}
#endif
