/*
 * Time loops: fmd_dync_integrate / fmd_dync_equilibrate.
 *
 * Control flow of the reference (src/integrators.c:181-325, timer events
 * src/timer.c:27-84) is kept on the host: the same FP64 time accumulation
 * `time += dt` under `while (time < start + duration)`, the same timer test
 * |t - tc| < dt/2, the same event order.  The per-step work runs on the GPU.
 * Steps between two host-visible events are issued as one batch of
 * graph launches without synchronisation; the host only waits when an
 * event handler runs (the handler may read state) or when the run ends.
 */
#include <math.h>
#include <stdlib.h>
#include "fmd_private.h"

#define FMD_MAX_BATCH (1 << 20)

fmd_real_t fmd_dync_getTimestep(fmd_t *md) { return md->timestep; }
fmd_real_t fmd_dync_getTime(fmd_t *md) { return md->time; }

static bool is_its_time(double t, double dt_half, double start, double interval)
{
    const double tc = round((t - start) / interval) * interval + start;
    const double d = t - tc;
    return d >= -dt_half && d < dt_half;
}

static bool timer_due(const fmd_t *md, const fmd_timer_t *tm, double t)
{
    return tm->enabled && (t >= tm->start - md->timestep / 2.0) &&
           ((t < tm->stop + md->timestep / 2.0) || tm->stop < tm->start) &&
           is_its_time(t, md->timestep / 2.0, tm->start, tm->interval);
}

static bool any_timer_due(const fmd_t *md, double t)
{
    for (int i = 0; i < md->timers_num; i++)
        if (timer_due(md, &md->timers[i], t)) return true;
    return false;
}

void _fmdh_send_timer_events(fmd_t *md)
{
    for (int i = 0; i < md->timers_num; i++)
        if (timer_due(md, &md->timers[i], md->time))
        {
            fmd_event_params_timer_tick_t p;
            p.timer = i;
            md->EventHandler(md, FMD_EVENT_TIMER_TICK, md->userobject, (fmd_params_t *)&p);
        }
}

/* device error bits become the reference's error events */
void _fmdh_check_device_errors(fmd_t *md)
{
    unsigned bits = 0;
    if (!_fmdh_dev_ok(md, fmdg_get_errors(md->dev, &bits, 1), "fmdg_get_errors")) return;
    if (bits & FMDG_ERRBIT_POSITION)
        FMD_ERR(md, FMD_ERR_UNEXPECTED_POSITION, true, "an atom moved beyond the neighbouring cell");
    if (bits & FMDG_ERRBIT_RHO_RANGE)
        FMD_ERR(md, FMD_ERR_OUTSIDE_REAL_INTERVAL, true,
                "electron density outside the interval of the EAM potential");
    if (bits & FMDG_ERRBIT_INTERNAL)
        FMD_ERR(md, FMD_ERR_FUNCTION_FAILED, true, "device engine index check failed");
    if (bits & FMDG_ERRBIT_TTM)
        FMD_ERR(md, FMD_ERR_UNEXPECTED_POSITION, true, "atom outside the turi grid");
    if (bits & FMDG_ERRBIT_TTM_TABLE)
        FMD_ERR(md, FMD_ERR_OUTSIDE_REAL_INTERVAL, true,
                "electron temperature outside the tabulated interval of the TTM");
}

static void set_active_group(fmd_t *md, int GroupID)
{
    if (GroupID != md->ActiveGroup)
    {
        md->ActiveGroup = GroupID;
        md->KineticEnergyUpdated = false;
    }
}

static bool prepare_run(fmd_t *md, int GroupID, double timestep)
{
    if (!_fmdh_distribute(md)) return false;
    if (!_fmdh_pots_ready(md)) return false;
    if (!_fmdh_dev_ok(md, _fmdh_upload_tables(md), "upload tables")) return false;
    set_active_group(md, GroupID);
    md->timestep = timestep;
    return true;
}

/* initial force evaluation of a run; leaves PE and the current kinetic
   terms in the device thermo record */
static bool initial_forces(fmd_t *md)
{
    if (!_fmdh_dev_ok(md, fmdg_compute_forces(md->dev, md->ActiveGroup), "fmdg_compute_forces")) return false;
    md->thermo_pending = true;
    md->KineticEnergyUpdated = true;
    return true;
}

/* velocity Verlet with optional Berendsen scaling (src/integrators.c:227-264) */
static void vv_integrate(fmd_t *md, double duration, bool thermostat)
{
    const double start = md->time;
    const double dt = md->timestep;
    const double tau = thermostat ? md->BerendsenThermostatParam : 1.0;
    const double T0 = thermostat ? md->DesiredTemperature : 0.0;
    if (md->turies_num > 0)
    {
        if (!_fmdh_prepare_turies(md)) return;
        if (!_fmdh_dev_ok(md, fmdg_set_time(md->dev, md->time, dt), "fmdg_set_time")) return;
    }
    if (!initial_forces(md)) return;
    unsigned due = 0;
    if (md->turies_num > 0)
    {
        due = _fmdh_turies_due(md);
        if (due && !_fmdh_dev_ok(md, fmdg_turi_update(md->dev, dt, due), "fmdg_turi_update")) return;
    }
    if (thermostat &&
        !_fmdh_dev_ok(md, fmdg_prepare_thermostat(md->dev, md->ActiveGroup, dt, tau, T0), "thermostat"))
        return;
    if (md->turies_num > 0) _fmdh_turies_updated(md, due, false);
    _fmdh_check_device_errors(md);
    if (md->EventHandler != NULL) _fmdh_send_timer_events(md);
    while (md->time < start + duration)
    {
        int k = 0;
        double t = md->time;
        do
        {
            k++;
            t += dt;
        } while (k < FMD_MAX_BATCH && t < start + duration && md->turies_num == 0 &&
                 !(md->EventHandler != NULL && any_timer_due(md, t)));
        if (!_fmdh_dev_ok(md, fmdg_vv_steps(md->dev, k, dt, md->ActiveGroup, thermostat ? 1 : 0, tau, T0),
                          "fmdg_vv_steps"))
            return;
        for (int s = 0; s < k; s++)
        {
            md->time += dt;
            md->time_iteration++;
        }
        md->thermo_pending = true;
        md->KineticEnergyUpdated = true;
        if (md->turies_num > 0) _fmdh_turies_update(md, true, true, true);
        _fmdh_check_device_errors(md);
        if (md->EventHandler != NULL) _fmdh_send_timer_events(md);
    }
}

void fmd_dync_integrate(fmd_t *md, int GroupID, fmd_real_t duration, fmd_real_t timestep)
{
    if (!prepare_run(md, GroupID, timestep)) return;
    if (md->active_ttm_turi != NULL)
    {
        /* symplectic Euler under TTM coupling (src/integrators.c:181-225) */
        _fmdh_se_integrate(md, duration);
        return;
    }
    vv_integrate(md, duration, false);
}

void fmd_dync_equilibrate(fmd_t *md, int GroupID, fmd_real_t duration, fmd_real_t timestep,
                          fmd_real_t tau, fmd_real_t temperature)
{
    if (!_fmdh_distribute(md)) return;
    const double bak_time = md->time;
    md->time = 0.0;
    md->DesiredTemperature = temperature;
    md->BerendsenThermostatParam = tau;
    if (!prepare_run(md, GroupID, timestep)) { md->time = bak_time; return; }
    vv_integrate(md, duration, true);
    md->time = bak_time;
}
