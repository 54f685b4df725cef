/* Empty stand-in for the PGPLOT C header.  The reference's samodel.c includes
 * it through samodelgraphics.h, but no PGPLOT symbol is referenced on the
 * inversion path (plotting is compiled out with PLOTTING 0). */
