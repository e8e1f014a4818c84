// st_ext.cu -- freeing the photon map's and the optics bench's device state with the context.
#include "st_ext.h"

void ext_free(StExt& e) {
    SppmState& s = e.sppm;
    void* ps[] = {s.pos, s.power, s.dir_oct, s.nrm_oct, s.flags, s.key, s.order, s.cell_count, s.cell_start,
                  s.heads, s.scan_part, s.spos, s.spow, s.sdir, s.snrm, s.sflags, s.stats, s.bucket, s.rank, (void*)s.dev,
                  s.lt_emit, s.lt_hit, s.lt_cdf};
    for (void* p : ps)
        if (p) cudaFree(p);
    GuideState& g = e.guide;
    void* gs[] = {g.param, g.grad, g.m1, g.m2, g.wbf, (void*)g.dev, (void*)g.samp, g.act, g.mix, (void*)g.stamp,
                  (void*)g.rec, g.acc};
    for (void* p : gs)
        if (p) cudaFree(p);
    EmitState& m = e.emit;
    void* ms[] = {m.grid, (void*)m.dev, m.w, m.hpos, m.hdir, m.hrad};
    for (void* p : ms)
        if (p) cudaFree(p);
    optics_free(e.optics);
    e = StExt{};
}
