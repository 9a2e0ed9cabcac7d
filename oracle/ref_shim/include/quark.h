/* Host stand-in for the QUARK runtime interface used by the reference's oocquark.cpp and
 * oocdag.cpp (QUARK itself is an un-vendored dependency, version unpinned).
 *
 * TEST INFRASTRUCTURE ONLY: lets the reference's own task generators and task bodies
 * compile and run on the host so that their output checks the oracle.  Semantics kept:
 * QUARK_Insert_Task packs (size, pointer, mode) triples; a VALUE argument is copied by
 * value, any other mode passes the pointer; quark_unpack_args_N copies the packed
 * arguments back in order.  Scheduling: every task runs at insertion, in program order,
 * which is one legal QUARK schedule (QUARK orders tasks by their declared data
 * hazards, so any schedule it picks gives the program-order result).  Task flags
 * (colour, label, priority, thread masks) only steer QUARK's placement and are
 * recorded, not used. */
#ifndef OOC_REF_SHIM_QUARK_H
#define OOC_REF_SHIM_QUARK_H

#include <stdint.h>
#include <string.h>

typedef struct ooc_shim_quark Quark;

typedef struct Quark_Task_Flags {
  intptr_t color, label, priority, thread_mask, thread;
} Quark_Task_Flags;
#define Quark_Task_Flags_Initializer {0, 0, 0, 0, -1}

enum { TASK_COLOR = 1, TASK_LABEL, TASK_PRIORITY, TASK_LOCK_TO_THREAD_MASK, TASK_LOCK_TO_THREAD };
enum { VALUE = 1, INPUT = 2, OUTPUT = 4, INOUT = 6, LOCALITY = 8 };

#ifdef __cplusplus
extern "C" {
#endif
Quark* QUARK_New(int nthreads);
void QUARK_Delete(Quark* q);
void QUARK_Barrier(Quark* q);
int QUARK_Thread_Rank(Quark* q);
void QUARK_DOT_DAG_Enable(Quark* q, int enable);
int quark_getenv_int(const char* name, int dflt);
Quark_Task_Flags* QUARK_Task_Flag_Set(Quark_Task_Flags* f, int flag, intptr_t val);
unsigned long long QUARK_Insert_Task(Quark* q, void (*fn)(Quark*), Quark_Task_Flags* f, ...);
/* the packed arguments of the task now running */
const unsigned char* ooc_shim_task_args(Quark* q);
#ifdef __cplusplus
}
#endif

#define OOC_SHIM_UNPACK_(p, a) memcpy(&(a), (p), sizeof(a)); (p) += sizeof(a);
#define quark_unpack_args_4(q, a1, a2, a3, a4) \
  { const unsigned char* _p = ooc_shim_task_args(q); OOC_SHIM_UNPACK_(_p, a1) OOC_SHIM_UNPACK_(_p, a2) OOC_SHIM_UNPACK_(_p, a3) OOC_SHIM_UNPACK_(_p, a4) }
#define quark_unpack_args_6(q, a1, a2, a3, a4, a5, a6) \
  { const unsigned char* _p = ooc_shim_task_args(q); OOC_SHIM_UNPACK_(_p, a1) OOC_SHIM_UNPACK_(_p, a2) OOC_SHIM_UNPACK_(_p, a3) OOC_SHIM_UNPACK_(_p, a4) OOC_SHIM_UNPACK_(_p, a5) OOC_SHIM_UNPACK_(_p, a6) }
#define quark_unpack_args_9(q, a1, a2, a3, a4, a5, a6, a7, a8, a9) \
  { const unsigned char* _p = ooc_shim_task_args(q); OOC_SHIM_UNPACK_(_p, a1) OOC_SHIM_UNPACK_(_p, a2) OOC_SHIM_UNPACK_(_p, a3) OOC_SHIM_UNPACK_(_p, a4) OOC_SHIM_UNPACK_(_p, a5) OOC_SHIM_UNPACK_(_p, a6) OOC_SHIM_UNPACK_(_p, a7) OOC_SHIM_UNPACK_(_p, a8) OOC_SHIM_UNPACK_(_p, a9) }
#define quark_unpack_args_10(q, a1, a2, a3, a4, a5, a6, a7, a8, a9, a10) \
  { const unsigned char* _p = ooc_shim_task_args(q); OOC_SHIM_UNPACK_(_p, a1) OOC_SHIM_UNPACK_(_p, a2) OOC_SHIM_UNPACK_(_p, a3) OOC_SHIM_UNPACK_(_p, a4) OOC_SHIM_UNPACK_(_p, a5) OOC_SHIM_UNPACK_(_p, a6) OOC_SHIM_UNPACK_(_p, a7) OOC_SHIM_UNPACK_(_p, a8) OOC_SHIM_UNPACK_(_p, a9) OOC_SHIM_UNPACK_(_p, a10) }
#define quark_unpack_args_11(q, a1, a2, a3, a4, a5, a6, a7, a8, a9, a10, a11) \
  { const unsigned char* _p = ooc_shim_task_args(q); OOC_SHIM_UNPACK_(_p, a1) OOC_SHIM_UNPACK_(_p, a2) OOC_SHIM_UNPACK_(_p, a3) OOC_SHIM_UNPACK_(_p, a4) OOC_SHIM_UNPACK_(_p, a5) OOC_SHIM_UNPACK_(_p, a6) OOC_SHIM_UNPACK_(_p, a7) OOC_SHIM_UNPACK_(_p, a8) OOC_SHIM_UNPACK_(_p, a9) OOC_SHIM_UNPACK_(_p, a10) OOC_SHIM_UNPACK_(_p, a11) }

#endif
