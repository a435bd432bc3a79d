/* Declaration-only stand-in for the assimp C API names that the reference's
 * main.h mentions; nothing here is ever called by the pin harness. */
#ifndef QPSO_PIN_ASSIMP_STUB_H
#define QPSO_PIN_ASSIMP_STUB_H
struct aiVector3D { float x, y, z; };
struct aiFace { unsigned int mNumIndices; unsigned int *mIndices; };
struct aiMesh { unsigned int mNumFaces; aiFace *mFaces; aiVector3D *mVertices; };
struct aiScene { aiMesh **mMeshes; };
#define aiProcessPreset_TargetRealtime_Fast 0
const aiScene *aiImportFile(const char *path, unsigned int flags);
#endif
