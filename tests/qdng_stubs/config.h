// Configuration of a QDng build as its autotools would write it, for the
// module compile check: dynamic modules on, no MPI.
#define HAVE_STRING_H 1
#define USE_DYNMODS 1
