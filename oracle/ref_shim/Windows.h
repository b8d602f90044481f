// TEST INFRASTRUCTURE ONLY -- stand-in for <Windows.h>, used only when the
// reference's own CPU sources are compiled as a second oracle.  The
// reference's IC-GN source includes its stopwatch header, whose class holds
// two LARGE_INTEGER members; nothing on the compiled path calls the Win32
// timer functions.
#ifndef TWREF_WINDOWS_STANDIN_H
#define TWREF_WINDOWS_STANDIN_H

typedef union {
    long long QuadPart;
} LARGE_INTEGER;

#endif
