/*
 * Test infrastructure only: the four documented sqlite3 C API calls the
 * reference uses, declared so it links against the runtime-only
 * libsqlite3.so.0 on the build host.
 */
#pragma once
#ifdef __cplusplus
extern "C" {
#endif
typedef struct sqlite3 sqlite3;
#define SQLITE_OK 0
int sqlite3_open(const char *filename, sqlite3 **db);
int sqlite3_close(sqlite3 *db);
const char *sqlite3_errmsg(sqlite3 *db);
int sqlite3_exec(sqlite3 *db, const char *sql,
                 int (*callback)(void *, int, char **, char **), void *arg,
                 char **errmsg);
#ifdef __cplusplus
}
#endif
