/* No-op definitions of the PGPLOT C routines the reference's plotting
 * objects (model/graphics.c, colours.c, plot.c, samodelgraphics.c) call, so
 * that the relink test can link the reference's whole program without the
 * PGPLOT library, which is not installed here.  Never called: the test only
 * links.  (The reference's graphics sources see an empty cpgplot.h, so
 * their calls carry implicit declarations; these definitions only have to
 * exist.) */
void cpgbbuf(void) {}
void cpgbox(void) {}
void cpgclos(void) {}
void cpgdraw(void) {}
void cpgebuf(void) {}
void cpgenv(void) {}
void cpglab(void) {}
void cpgmove(void) {}
int cpgopen(void) { return 0; }
void cpgpap(void) {}
void cpgpt1(void) {}
void cpgrect(void) {}
void cpgsch(void) {}
void cpgsci(void) {}
void cpgscir(void) {}
void cpgscr(void) {}
void cpgsls(void) {}
void cpgslw(void) {}
void cpgsubp(void) {}
void cpgwedg(void) {}
