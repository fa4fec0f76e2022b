// Oracle test infrastructure: the few Win32 type names that the reference's window and
// camera headers mention. No Win32 function is declared or called by the oracle build.
#pragma once
#include <cstdint>
typedef void* HWND;
typedef void* HDC;
typedef void* HBITMAP;
typedef void* HINSTANCE;
typedef long LRESULT;
typedef unsigned int UINT;
typedef std::uintptr_t WPARAM;
typedef std::intptr_t LPARAM;
#ifndef CALLBACK
#define CALLBACK
#endif
