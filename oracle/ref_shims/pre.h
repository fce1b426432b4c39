/* Pre-include for compiling the reference's own sources headless (oracle
 * build only): CImg without display or TIFF, the utilities vec3, and the
 * imagelist typedef that WaP_Tomo.cpp expects. */
#define cimg_display 0
#include <functional>
#include <algorithm>
#include <cstring>
#include "CImg.h"
#include <vec3.h>
#include <iostream>
/* The reference relies on MSVC's lookup of unqualified std names inside
 * templates and on an `imagelist` typedef declared after its first use. */
using namespace std;
typedef cimg_library::CImgList<float> imagelist;
#include <cstdlib>
/* PSART::Render ends the process with exit(0); the oracle harness turns that
 * into an exception so the caller regains control after one Render pass. */
struct wap_ref_exit_signal { int code; };
[[noreturn]] inline void wap_ref_exit_hook(int code) { throw wap_ref_exit_signal{code}; }
#define exit(code) wap_ref_exit_hook(code)
