/*
 * argon_relink.c -- a caller of the fmd.h API written the way FMD's own
 * argon example is (examples/01_argon.c): an event handler with two simple
 * timers (one prints temperature and total energy, one saves the
 * configuration), an argon FCC box with periodic faces, a 12-6
 * Lennard-Jones potential with cutoff 2.5 sigma, a Berendsen equilibration
 * at 100 K with dt = 2 fs and tau = 0.02 ps, the final state saved and the
 * instance freed.  Two changes make it deterministic and single-process:
 * the initial state comes from a state file (argv[1]; the reference seeds
 * its velocity generator from the wall clock) and one subdomain is used.
 * Output files go to argv[2].  The same source is compiled unchanged
 * against the reference's fmd.h (golden run) and this library's
 * include/fmd.h (test), and linked with -lfmd.
 *
 *   gcc -std=c11 argon_relink.c -I<include> -L<lib> -lfmd -o argon_relink
 *   ./argon_relink state.stt outdir/ [duration_ps]
 */
#include <stdio.h>
#include <stdlib.h>
#include <fmd.h>

static fmd_handle_t timer1, timer2;

static void handleEvents(fmd_t *md, fmd_event_t event, void *usp, fmd_params_t *params)
{
    (void)usp;
    if (event != FMD_EVENT_TIMER_TICK) return;
    fmd_handle_t timer = ((fmd_event_params_timer_tick_t *)params)->timer;
    if (timer == timer1)
        printf("tick %.17g %.17g %.17g\n", fmd_dync_getTime(md), fmd_matt_getTemperature(md),
               fmd_matt_getTotalEnergy(md));
    else if (timer == timer2)
        fmd_matt_saveConfiguration(md);
}

int main(int argc, char **argv)
{
    if (argc < 3)
    {
        fprintf(stderr, "usage: %s state.stt outdir/ [duration_ps]\n", argv[0]);
        return 2;
    }
    const double duration = argc > 3 ? atof(argv[3]) : 0.4;
    fmd_t *md = fmd_create();
    fmd_setEventHandler(md, &md, handleEvents);
    timer1 = fmd_timer_makeSimple(md, 0.0, 0.05, -1.0);
    timer2 = fmd_timer_makeSimple(md, 0.0, 0.2, -1.0);
    const double LatticeParameter = 5.26;
    fmd_box_setSize(md, 10 * LatticeParameter, 10 * LatticeParameter, 10 * LatticeParameter);
    fmd_box_setPBC(md, true, true, true);
    if (!fmd_box_setSubdomains(md, 1, 1, 1)) return 3;
    fmd_string_t name[1] = {"Ar"};
    double mass[1] = {39.948};
    fmd_matt_setAtomKinds(md, 1, name, mass);
    const double sigma = 3.4, epsilon = 0.0104;
    fmd_pot_lj_apply(md, 0, 0, sigma, epsilon, 2.5 * sigma);
    fmd_io_setSaveDirectory(md, argv[2]);
    fmd_io_setSaveConfigMode(md, FMD_SCM_XYZ_ATOMSNUM);
    fmd_io_loadState(md, argv[1], false);
    fmd_dync_equilibrate(md, 0, duration, 2e-3, 2e-2, 100.0);
    fmd_io_saveState(md, "state1.stt");
    printf("done %.17g %u\n", fmd_dync_getTime(md), fmd_matt_getTotalEnergy(md) < 0.0);
    fmd_free(md);
    return 0;
}
