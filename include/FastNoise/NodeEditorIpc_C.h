/* NodeEditorIpc_C.h -- the FastNoise2 Node Editor's shared-memory channel, as exported by
 * libfastnoise_gb300.so.
 *
 * Same entry points, message codes and wire format as the reference's NodeEditorIpc library
 * (tools/NodeEditorIpc/include/FastNoise/NodeEditorIpc_C.h:10-66, implementation
 * tools/NodeEditorIpc/NodeEditorIpc_C.cpp), so an application linked against this library and
 * a running FastNoise2 Node Editor exchange encoded node trees with each other: a POSIX shared
 * memory object "/FastNoise2NodeEditor" of 64 KiB holding a message counter (byte 0), the
 * message type (byte 1) and a NUL-terminated encoded node tree (from byte 2).
 *
 * Live trees (fnLiveTree*, declared in FastNoise_C.h) build on this channel: they follow the
 * trees the editor sends and swap them into generation and serving without a pause.
 */
#ifndef FASTNOISE_GB300_NODEEDITORIPC_C_H
#define FASTNOISE_GB300_NODEEDITORIPC_C_H

#ifndef FASTNOISE_API
#if defined(_WIN32)
#define FASTNOISE_API __declspec(dllexport)
#else
#define FASTNOISE_API __attribute__((visibility("default")))
#endif
#endif

#ifdef __cplusplus
extern "C" {
#else
#include <stdbool.h>
#endif

/* Message types / return codes (NodeEditorIpc_C.h:10-15) */
#define FASTNOISE_EDITORIPC_MSG_IPC_NOT_INITIALISED (-2)
#define FASTNOISE_EDITORIPC_MSG_BUFFER_TOO_SMALL    (-1)
#define FASTNOISE_EDITORIPC_MSG_NONE                  0
#define FASTNOISE_EDITORIPC_MSG_SELECTED_NODE         1   /* the editor's selected / modified tree */
#define FASTNOISE_EDITORIPC_MSG_IMPORT_REQUEST        2   /* a tree for the editor to import */

/* Open (creating if needed) the shared channel.  readPrevious: the first poll also returns a
 * selected-node message already waiting in the channel.  NULL on failure (:17-22). */
FASTNOISE_API void* fnEditorIpcSetup(bool readPrevious);

/* Unmap the channel and remove its name (:24-28). */
FASTNOISE_API void fnEditorIpcRelease(void* ipc);

/* Publish a selected tree, as the editor does when the user selects or edits a node; false
 * when the context is NULL or the string does not fit in the channel (:30-36). */
FASTNOISE_API bool fnEditorIpcSendSelectedNode(void* ipc, const char* encodedNodeTree);

/* Ask the editor to import a tree into its node graph (:38-44). */
FASTNOISE_API bool fnEditorIpcSendImportRequest(void* ipc, const char* encodedNodeTree);

/* The newest message not yet seen by this context (messages this context sent are skipped):
 * its type with the tree copied into outBuffer, FASTNOISE_EDITORIPC_MSG_NONE when nothing new,
 * _BUFFER_TOO_SMALL, or _IPC_NOT_INITIALISED for a NULL context (:46-53). */
FASTNOISE_API int fnEditorIpcPollMessage(void* ipc, char* outBuffer, int bufferSize);

/* Path of the NodeEditor executable for fnEditorIpcStartNodeEditor; NULL clears it (:55-59). */
FASTNOISE_API void fnEditorIpcSetNodeEditorPath(const char* path);

/* Start a NodeEditor process: the path set above, else "NodeEditor" next to this library or in
 * ../bin from it, else ./NodeEditor, ../bin/NodeEditor, ./bin/NodeEditor.  Arguments
 * "--detached" (node graph only) and "--import-ent <tree>".  childProcess = false starts it in
 * its own session.  false when no executable was found or it could not be started (:61-67). */
FASTNOISE_API bool fnEditorIpcStartNodeEditor(const char* encodedNodeTree, bool detached, bool childProcess);

#ifdef __cplusplus
}
#endif

#endif
