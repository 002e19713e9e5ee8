// Test-side harness around the reference's own input reader.
//
// Test infrastructure only: links Input::readinfo (src/IO/readinfo.cpp) and
// Input::ProcessInfo (src/IO/check.cpp), compiled in place from the
// reference sources, with libconfig 1.5 compiled from the tarball the
// reference ships (oracle/ref/Makefile), and exposes them as a flat C ABI so
// the tests can compare the library's emoo_read_input / emoo_process_info
// with the reference byte for byte on the same input files.
// the reference's globals (rank, size_MPI, time_phys, ...) are defined where
// MAIN_CPP is set, in its driver; this library has no driver
#define MAIN_CPP
#include "globals.hpp"
#include <cstring>

#include "IO/input.hpp"

extern "C" {

// Input::readinfo on `path` into *out; the reference leaves members it does
// not set uninitialised (Input::Input news the struct), so the struct is
// zeroed first, as emoo_read_input does. Returns readinfo's status (0 = ok).
int refi_read_input(const char *path, Input_Info_t *out) {
    Input in;
    memset(in.getinfo(), 0, sizeof(Input_Info_t));
    int rc = in.readinfo(const_cast<char *>(path));
    memcpy(out, in.getinfo(), sizeof(Input_Info_t));
    return rc;
}

// Input::ProcessInfo on *info (in place). Returns its error count.
int refi_process_info(Input_Info_t *info) {
    Input in;
    memcpy(in.getinfo(), info, sizeof(Input_Info_t));
    int rc = in.ProcessInfo();
    memcpy(info, in.getinfo(), sizeof(Input_Info_t));
    return rc;
}

int refi_sizeof_input_info(void) { return (int)sizeof(Input_Info_t); }

}  // extern "C"
