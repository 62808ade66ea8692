/* diffuse-particle oracle: filled in with the diffuse stages */
