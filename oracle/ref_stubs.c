/* Link stubs for building the reference inversion path: nothing is needed
 * beyond oracle/ref_ncstub.c (the in-memory stand-in for libnetcdf that the
 * reference's own model/nc.c writes and reads through). */
typedef int photic_ref_stubs_translation_unit_is_not_empty;
