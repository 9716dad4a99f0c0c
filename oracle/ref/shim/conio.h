/* Linux stand-in for the Windows <conio.h> header; the reference's
 * console helpers only need these two names to compile.  Oracle build only. */
#pragma once
static inline int _kbhit(void) { return 0; }
static inline int _getch(void) { return 0; }
