/* Logging shim: the mlog submodule is not vendored; messages are dropped. */
#ifndef MXS_MLOG_H
#define MXS_MLOG_H
#define MLOG_MESG 1
#define MLOG_OPEN 2
#define MLOG_CLOSE 4
#define MLOG_CONT 8
#define MLOG_FLUSH 16
#define MLOG_TIMERSTART 32
#define MLOG_TIMERSTOP 64
#define MLOG_ALLRANKS 128
#define mlog(...) ((void)0)
#define mlog_error(...) ((void)0)
#endif
