/*
 * CPU worker: pops tasks from its dmda queue, brings their data to host RAM,
 * runs cpu_funcs[0] and reports the measured time to the history model
 * (src/drivers/cpu/driver_cpu.c:374 execute_job_on_cpu, and
 * src/drivers/driver_common/driver_common.c:43,172,234 for the timing and
 * feedback).
 */
#include "rt_internal.h"

static void run_cpu(struct rt_worker *w, struct rt_job *j)
{
    struct starpu_task *t = j->task;
    rt_lock();
    if (rt.relaxed_commute) rt_commute_acquire(t);
    for (int i = 0; i < t->nbuffers; ++i) {
        starpu_data_handle_t h = t->handles[i];
        if (!h) continue;
        int rc = rt_data_fetch(h, RT_NODE_RAM, t->modes[i], NULL);
        STARPU_ASSERT_MSG(rc == 0, "cannot fetch data %d of task %s to RAM (%d)", i, t->name ? t->name : "?", rc);
        t->interfaces[i] = rt_data_interface(h, RT_NODE_RAM);
    }
    rt_unlock();
    rt_current_task_set(t);
    double t0 = starpu_timing_now();
    if (t->cl && t->cl->cpu_funcs[0]) t->cl->cpu_funcs[0](t->interfaces, t->cl_arg);
    double us = starpu_timing_now() - t0;
    rt_current_task_set(NULL);
    rt_lock();
    for (int i = 0; i < t->nbuffers; ++i)
        if (t->handles[i] && (t->modes[i] & STARPU_W)) rt_data_after_write(t->handles[i], RT_NODE_RAM);
    if (rt.relaxed_commute) rt_commute_release(t);
    rt.stats.tasks_cpu++;
    w->ntasks++;
    rt_unlock();
    rt_job_terminate(j, us);
}

void *rt_cpu_worker_main(void *arg)
{
    struct rt_worker *w = arg;
    rt_set_current_worker(w->id);
    rt_lock();
    for (;;) {
        struct rt_job *j = NULL;
        while (!(j = rt_sched_pop(w))) {
            if (rt.shutting_down) {
                rt_unlock();
                return NULL;
            }
            pthread_cond_wait(&w->cond, &rt.lock);
        }
        rt_unlock();
        run_cpu(w, j);
        rt_lock();
    }
}
