// server_format.h -- message parsing and result rows of the reference's
// server surface (host only).
#pragma once
#include <string>

#include "../../include/scs.h"

#define SCS_MSG_MAX 80     /* ipc/msgtool.h:16 MAX_SEND_SIZE */
#define SCS_MSG_DIR "/tmp" /* ipc/msgtool.h:17 MSG_DIR */

// "server_exit" after trimming blanks, case-insensitive (main.cu:51-60)
bool scs_is_server_exit(const std::string &s);
// exactly five unsigned integers (main.cu:92-109)
bool scs_parse_query(const std::string &s, scs_query &q);
// 1,234,567 grouping of inc/Utility.h:72-90
std::string scs_group_thousands(long long v);
// one result row N1|N2|QID|Time|Degree|Overtime|Heu|TotalTime as the
// reference writes it for each outcome (main.cu:124-128, 328-333, 348-352,
// 451-454); Time is microseconds from submission
std::string scs_format_row(const scs_result &r);
